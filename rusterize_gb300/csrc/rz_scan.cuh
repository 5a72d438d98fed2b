// rz_scan.cuh -- exclusive prefix sums over K-column rows (reduce / scan /
// apply, recursive over block totals).  out has n+1 rows; out[n] = total.
#pragma once

#include <cuda_runtime.h>

namespace rzd {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr unsigned long long SCAN_TILE = (unsigned long long)SCAN_THREADS * SCAN_ITEMS;

// A block covers SCAN_TILE rows; warp w of the block takes its SCAN_WROWS
// consecutive rows 32 at a time (lane = row), so every load of a column is
// one coalesced sweep over 32 neighbouring rows, and a shuffle scan per
// group of 32 plus a running carry give the warp's prefixes.
constexpr int SCAN_WARPS = SCAN_THREADS / 32;
constexpr int SCAN_WROWS = (int)(SCAN_TILE / SCAN_WARPS);
constexpr int SCAN_GROUPS = SCAN_WROWS / 32;

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += t;
  }
  return x;
}

template <typename T, int K>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const T* __restrict__ in,
                                                              unsigned long long n, T* __restrict__ sums) {
  __shared__ T s_tot[SCAN_WARPS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned long long r0 = (unsigned long long)blockIdx.x * SCAN_TILE + (unsigned long long)warp * SCAN_WROWS;
  for (int k = 0; k < K; ++k) {
    T acc = 0;
#pragma unroll 4
    for (int gi = 0; gi < SCAN_GROUPS; ++gi) {
      const unsigned long long row = r0 + (unsigned long long)gi * 32 + lane;
      if (row < n) acc += in[row * K + k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    if (lane == 0) s_tot[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      T total = 0;
      for (int w = 0; w < SCAN_WARPS; ++w) total += s_tot[w];
      sums[(unsigned long long)blockIdx.x * K + k] = total;
    }
    __syncthreads();
  }
}

template <typename T, int K>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const T* __restrict__ in, unsigned long long n,
                                                             const T* __restrict__ block_off,
                                                             T* __restrict__ out) {
  __shared__ T s_tot[SCAN_WARPS];
  __shared__ T s_off[SCAN_WARPS + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned long long r0 = (unsigned long long)blockIdx.x * SCAN_TILE + (unsigned long long)warp * SCAN_WROWS;
  for (int k = 0; k < K; ++k) {
    T ex[SCAN_GROUPS];  // exclusive prefix of each of this lane's rows within the warp's rows
    T carry = 0;
#pragma unroll
    for (int gi = 0; gi < SCAN_GROUPS; ++gi) {
      const unsigned long long row = r0 + (unsigned long long)gi * 32 + lane;
      const T v = row < n ? in[row * K + k] : T(0);
      const T x = warp_inclusive_scan<T>(v);
      ex[gi] = carry + x - v;
      carry += __shfl_sync(0xFFFFFFFFu, x, 31);
    }
    if (lane == 0) s_tot[warp] = carry;
    __syncthreads();
    if (threadIdx.x == 0) {
      T run = 0;
      for (int w = 0; w < SCAN_WARPS; ++w) {
        s_off[w] = run;
        run += s_tot[w];
      }
      s_off[SCAN_WARPS] = run;
    }
    __syncthreads();
    const T boff = block_off ? block_off[(unsigned long long)blockIdx.x * K + k] : T(0);
    const T off = boff + s_off[warp];
#pragma unroll
    for (int gi = 0; gi < SCAN_GROUPS; ++gi) {
      const unsigned long long row = r0 + (unsigned long long)gi * 32 + lane;
      if (row < n) out[row * K + k] = off + ex[gi];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n * K + k] = boff + s_off[SCAN_WARPS];
    __syncthreads();  // s_tot / s_off are reused by the next column
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
