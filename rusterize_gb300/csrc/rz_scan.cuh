// rz_scan.cuh -- exclusive prefix sums over K-column rows (reduce / scan /
// apply, recursive over block totals).  out has n+1 rows; out[n] = total.
#pragma once

#include <cuda_runtime.h>

namespace rzd {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr unsigned long long SCAN_TILE = (unsigned long long)SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* s_warp, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = lane < SCAN_THREADS / 32 ? s_warp[lane] : T(0);
    T wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < SCAN_THREADS / 32) s_warp[lane] = wi - w;
    if (lane == SCAN_THREADS / 32 - 1) s_warp[32] = wi;
  }
  __syncthreads();
  T res = s_warp[warp] + incl - v;
  *total = s_warp[32];
  __syncthreads();
  return res;
}

template <typename T, int K>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const T* __restrict__ in,
                                                              unsigned long long n, T* __restrict__ sums) {
  __shared__ T s_warp[33];
  const unsigned long long base = (unsigned long long)blockIdx.x * SCAN_TILE;
  for (int k = 0; k < K; ++k) {
    T acc = 0;
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      unsigned long long row = base + (unsigned long long)i * SCAN_THREADS + threadIdx.x;
      if (row < n) acc += in[row * K + k];
    }
    T total;
    block_exclusive_scan<T>(acc, s_warp, &total);
    if (threadIdx.x == 0) sums[(unsigned long long)blockIdx.x * K + k] = total;
  }
}

template <typename T, int K>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const T* __restrict__ in, unsigned long long n,
                                                             const T* __restrict__ block_off,
                                                             T* __restrict__ out) {
  __shared__ T s_warp[33];
  const unsigned long long base = (unsigned long long)blockIdx.x * SCAN_TILE +
                                  (unsigned long long)threadIdx.x * SCAN_ITEMS;
  for (int k = 0; k < K; ++k) {
    T vals[SCAN_ITEMS];
    T sum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      unsigned long long row = base + i;
      vals[i] = row < n ? in[row * K + k] : T(0);
      sum += vals[i];
    }
    T total;
    T run = block_exclusive_scan<T>(sum, s_warp, &total);
    T off = block_off ? block_off[(unsigned long long)blockIdx.x * K + k] : T(0);
    run += off;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      unsigned long long row = base + i;
      if (row < n) out[row * K + k] = run;
      run += vals[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n * K + k] = off + total;
  }
}

// Scratch elements (of T) needed by scan() for n rows of K columns.
inline unsigned long long scan_temp_elems(unsigned long long n, int K) {
  unsigned long long need = 0;
  while (true) {
    unsigned long long nblk = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nblk <= 1) break;
    need += (2 * nblk + 1) * (unsigned long long)K;
    n = nblk;
  }
  return need + 1;
}

// Returns the number of kernel launches issued.
template <typename T, int K>
int scan(const T* in, T* out, unsigned long long n, T* temp, cudaStream_t s) {
  unsigned long long nblk = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nblk == 0) nblk = 1;
  if (nblk == 1) {
    k_scan_apply<T, K><<<1, SCAN_THREADS, 0, s>>>(in, n, nullptr, out);
    return 1;
  }
  T* sums = temp;
  T* sums_out = temp + nblk * K;
  T* next = sums_out + (nblk + 1) * K;
  k_scan_reduce<T, K><<<(unsigned)nblk, SCAN_THREADS, 0, s>>>(in, n, sums);
  int launches = 1 + scan<T, K>(sums, sums_out, nblk, next, s);
  k_scan_apply<T, K><<<(unsigned)nblk, SCAN_THREADS, 0, s>>>(in, n, sums_out, out);
  return launches + 1;
}

}  // namespace rzd
