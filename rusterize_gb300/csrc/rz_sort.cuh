// rz_sort.cuh -- stable least-significant-digit radix sort of (64-bit key,
// 32-bit value) pairs, 8 bits per pass: a per-tile digit histogram, one
// exclusive scan of the digit-major histogram table, and a scatter that ranks
// every element inside its tile stably (tile rounds in index order, ranks
// within a warp from __match_any_sync, warp prefixes in shared memory).
#pragma once

#include <cuda_runtime.h>

#include "rz_scan.cuh"

namespace rzd {

constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 4;
constexpr unsigned RS_TILE = RS_THREADS * RS_ROUNDS;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned long long* __restrict__ keys, unsigned n,
                                                         int shift, unsigned* __restrict__ hist, unsigned nblocks) {
  __shared__ unsigned s_h[256];
  s_h[threadIdx.x] = 0u;
  __syncthreads();
  const unsigned base = blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const unsigned e = base + r * RS_THREADS + threadIdx.x;
    if (e < n) atomicAdd(&s_h[(unsigned)(keys[e] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * nblocks + blockIdx.x] = s_h[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const unsigned long long* __restrict__ kin,
                                                            const unsigned* __restrict__ vin,
                                                            unsigned long long* __restrict__ kout,
                                                            unsigned* __restrict__ vout, unsigned n, int shift,
                                                            const unsigned* __restrict__ off, unsigned nblocks) {
  __shared__ unsigned s_w[RS_THREADS / 32][256];  // per-warp digit counts, then warp prefixes
  __shared__ unsigned s_run[256], s_tot[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  s_run[threadIdx.x] = 0u;
  const unsigned base = blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ROUNDS; ++r) {
#pragma unroll
    for (int w = 0; w < RS_THREADS / 32; ++w) s_w[w][threadIdx.x] = 0u;
    __syncthreads();
    const unsigned e = base + r * RS_THREADS + threadIdx.x;
    const bool valid = e < n;
    unsigned long long k = 0;
    unsigned v = 0;
    if (valid) {
      k = kin[e];
      v = vin[e];
    }
    const unsigned d = valid ? (unsigned)(k >> shift) & 255u : 256u + (unsigned)lane;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    const unsigned rank = (unsigned)__popc(peers & lt);
    if (valid && rank == 0) s_w[warp][d] = (unsigned)__popc(peers);
    __syncthreads();
    {  // thread t = digit t: exclusive prefix over the warps, in warp order
      unsigned acc = 0;
#pragma unroll
      for (int w = 0; w < RS_THREADS / 32; ++w) {
        const unsigned c = s_w[w][threadIdx.x];
        s_w[w][threadIdx.x] = acc;
        acc += c;
      }
      s_tot[threadIdx.x] = acc;
    }
    __syncthreads();
    if (valid) {
      const unsigned pos = off[d * nblocks + blockIdx.x] + s_run[d] + s_w[warp][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
    s_run[threadIdx.x] += s_tot[threadIdx.x];
  }
}

// Scratch (in 32-bit words) for radix_sort on n elements.
inline unsigned long long radix_sort_temp_words(unsigned long long n) {
  const unsigned long long nblocks = (n + RS_TILE - 1) / RS_TILE;
  const unsigned long long h = 256ull * (nblocks ? nblocks : 1);
  return 2 * h + 1 + scan_temp_elems(h, 1);
}

// Sort keys[0..n) (bits [0, bits) significant) carrying vals; ktmp / vtmp are
// buffers of n elements.  Returns true when the sorted data ended up in
// ktmp / vtmp.  `launches` counts the kernels issued.
inline bool radix_sort(unsigned long long* keys, unsigned* vals, unsigned long long* ktmp, unsigned* vtmp, unsigned n,
                       int bits, unsigned* temp, cudaStream_t s, int& launches) {
  if (n == 0) return false;
  const unsigned nblocks = (n + RS_TILE - 1) / RS_TILE;
  const unsigned long long h = 256ull * nblocks;
  unsigned* hist = temp;
  unsigned* hoff = temp + h;
  unsigned* stmp = temp + 2 * h + 1;
  bool in_tmp = false;
  for (int shift = 0; shift < bits; shift += 8) {
    const unsigned long long* kin = in_tmp ? ktmp : keys;
    const unsigned* vin = in_tmp ? vtmp : vals;
    unsigned long long* kout = in_tmp ? keys : ktmp;
    unsigned* vout = in_tmp ? vals : vtmp;
    k_rs_hist<<<nblocks, RS_THREADS, 0, s>>>(kin, n, shift, hist, nblocks);
    launches += 1 + scan<unsigned, 1>(hist, hoff, h, stmp, s);
    k_rs_scatter<<<nblocks, RS_THREADS, 0, s>>>(kin, vin, kout, vout, n, shift, hoff, nblocks);
    ++launches;
    in_tmp = !in_tmp;
  }
  return in_tmp;
}

}  // namespace rzd
