// rz_sparse.cuh -- the sparse (COO) encoding: coverage records ordered by
// (band, part, row, word) and expanded into (row, col, value) triplets, one
// per written pixel (SparseArrayWriter, rust/src/encoding/writers.rs:86-131).
#pragma once

#include <type_traits>

#include "rz_device.cuh"

namespace rzd {

// sort keys of the parts by band (part order kept within a band)
__global__ void k_part_band_keys(const PartPlan* __restrict__ plan, unsigned long long P, unsigned long long* keys,
                                 unsigned* vals) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < P; p += stride) {
    keys[p] = ((unsigned long long)plan[p].band << 32) | p;
    vals[p] = (unsigned)p;
  }
}

__global__ void k_part_rank(const unsigned* __restrict__ sorted_parts, unsigned long long P, unsigned* prank) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < P; i += stride)
    prank[sorted_parts[i]] = (unsigned)i;
}

// key = band-major part rank << 32 | word id within the band's raster
__global__ void k_rec_keys(RecBuf rb, unsigned long long n, const unsigned* __restrict__ prank,
                           const PartPlan* __restrict__ plan, unsigned long long* keys, unsigned* vals) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const unsigned part = rb.part[i] & REC_PART_MASK;
    const unsigned pr = prank ? prank[part] : part;
    keys[i] = ((unsigned long long)pr << 32) | (rb.wid[i] - plan[part].wid0);
    vals[i] = (unsigned)i;
  }
}

// pixels each ordered record writes: a deduplicating part writes a pixel of
// a word once (its records of one word are adjacent in the order)
__global__ void k_sparse_count(const unsigned long long* __restrict__ skeys, const unsigned* __restrict__ svals,
                               unsigned long long n, RecBuf rb, unsigned* eff, unsigned long long* counts) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const unsigned rec = svals[i];
    unsigned m = rb.mask[rec];
    if (rb.part[rec] & DEDUP_BIT) {
      unsigned before = 0u;
      for (unsigned long long j = i; j > 0 && skeys[j - 1] == skeys[i]; --j) before |= rb.mask[svals[j - 1]];
      m &= ~before;
    }
    eff[i] = m;
    counts[i] = (unsigned long long)__popc(m);
  }
}

template <int VB>
__global__ void k_sparse_emit(const unsigned long long* __restrict__ skeys, const unsigned* __restrict__ svals,
                              unsigned long long n, RecBuf rb, const unsigned* __restrict__ eff,
                              const unsigned long long* __restrict__ offsets, const PartPlan* __restrict__ plan,
                              const void* __restrict__ values, const unsigned* __restrict__ part_geom,
                              unsigned long long scalar_bits, unsigned long long* rows, unsigned long long* cols,
                              void* tvals, unsigned long long* band_counts) {
  using V = typename std::conditional<VB == 1, unsigned char,
            typename std::conditional<VB == 2, unsigned short,
            typename std::conditional<VB == 4, unsigned, unsigned long long>::type>::type>::type;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    unsigned m = eff[i];
    if (!m) continue;
    const unsigned part = rb.part[svals[i]] & REC_PART_MASK;
    const unsigned lwid = (unsigned)skeys[i];
    const unsigned wpr = plan[part].wpr;
    const unsigned long long y = lwid / wpr;
    const unsigned long long x0 = (unsigned long long)(lwid % wpr) * 32u;
    const V v = values ? static_cast<const V*>(values)[part_geom[part]] : (V)scalar_bits;
    unsigned long long pos = offsets[i];
    atomicAdd(&band_counts[plan[part].band], (unsigned long long)__popc(m));
    while (m) {
      const unsigned b = (unsigned)(__ffs(m) - 1);
      m &= m - 1u;
      rows[pos] = y;
      cols[pos] = x0 + b;
      static_cast<V*>(tvals)[pos] = v;
      ++pos;
    }
  }
}

// ---- replay of a triplet stream (SparseArray::build_array) ----

// Key of every triplet of a chunk: the band comes from the band start
// offsets (bstart[b] <= t < bstart[b + 1] for stream index t), rows and
// columns are checked against the raster (the reference indexes the array and
// panics outside it; here the first bad stream index is reported).
__global__ void k_replay_keys(const unsigned long long* __restrict__ rows, const unsigned long long* __restrict__ cols,
                              unsigned n, unsigned long long t0, const unsigned long long* __restrict__ bstart,
                              unsigned n_bands, unsigned long long nrows, unsigned long long ncols,
                              unsigned long long* keys, unsigned* idx, Ctrl* ctrl) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long t = t0 + i;
    unsigned lo = 0, hi = n_bands - 1;  // the last band whose start is <= t
    while (lo < hi) {
      const unsigned mid = lo + (hi - lo + 1) / 2;
      if (bstart[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const unsigned long long r = rows[i], c = cols[i];
    unsigned long long key = 0;
    if (r < nrows && c < ncols) key = ((unsigned long long)lo * nrows + r) * ncols + c;
    else set_error(ctrl, ERR_TRIPLET, t);
    keys[i] = key;
    idx[i] = i;
  }
}

// Background of a raster of n elements of VB bytes.
template <int VB>
__global__ void k_replay_bg(void* p, unsigned long long n, unsigned long long bg) {
  using U = typename std::conditional<VB == 1, unsigned char,
            typename std::conditional<VB == 2, unsigned short,
            typename std::conditional<VB == 4, unsigned, unsigned long long>::type>::type>::type;
  U* q = static_cast<U*>(p);
  const U v = (U)bg;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    q[i] = v;
}

}  // namespace rzd
