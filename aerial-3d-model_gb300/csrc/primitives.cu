// Exclusive scan, stable LSD radix sort and batched lower_bound.
#include <vector>

#include "ba_common.cuh"
#include "primitives.cuh"

namespace ba {

thread_local int64_t g_launches = 0;


namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048

// Exclusive scan of one 2048-element tile; writes the tile total.
__global__ void __launch_bounds__(kScanThreads)
    scan_tile_kernel(const uint32_t* in, uint32_t* out, uint32_t* tile_sums,
                     size_t n) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    sum += v[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = (lane < kScanThreads / 32) ? warp_tot[lane] : 0u;
    uint32_t ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(kFull, ti, o);
      if (lane >= o) ti += u;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = ti - t;  // exclusive
    if (lane == kScanThreads / 32 - 1 && tile_sums) tile_sums[blockIdx.x] = ti;
  }
  __syncthreads();
  uint32_t run = warp_tot[warp] + incl - sum;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

__global__ void scan_add_kernel(uint32_t* out, const uint32_t* tile_off,
                                size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_off[i / kScanTile];
}

void scan_rec(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s) {
  const size_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles <= 1) {
    BA_LAUNCH(scan_tile_kernel<<<1, kScanThreads, 0, s>>>(in, out, nullptr, n));
    return;
  }
  DevBuf<uint32_t> sums(tiles, s);
  BA_LAUNCH(scan_tile_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, sums, n));
  scan_rec(sums, sums, tiles, s);
  BA_LAUNCH(scan_add_kernel<<<grid_for(n, 256), 256, 0, s>>>(out, sums, n));
}

// ---- radix sort ------------------------------------------------------------

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 2048
// 9-bit digits: the keys sorted here carry up to 18 bits (a destination block
// a * B + b of a few hundred block rows, a camera or point index), two passes.
constexpr int kRadixBits = 9;
constexpr int kRadix = 1 << kRadixBits;  // 512
constexpr int kPerThread = kRadix / kSortThreads;  // buckets per thread
static_assert(kRadix % kSortThreads == 0, "whole buckets per thread");

__global__ void __launch_bounds__(kSortThreads)
    radix_hist_kernel(const uint64_t* keys, size_t n, int shift,
                      uint32_t* hist, size_t ntiles) {
  __shared__ uint32_t cnt[kRadix];
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) cnt[threadIdx.x + j * kSortThreads] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kSortTile;
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i = base + (size_t)r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) {
    const int d = threadIdx.x + j * kSortThreads;
    hist[(size_t)d * ntiles + blockIdx.x] = cnt[d];
  }
}

// Stable scatter: items of one tile are ranked in index order, 256 at a time.
template <typename V>
__global__ void __launch_bounds__(kSortThreads)
    radix_scatter_kernel(const uint64_t* keys, const V* vals, uint64_t* okeys,
                         V* ovals, size_t n, int shift, const uint32_t* offs,
                         size_t ntiles) {
  __shared__ uint32_t base_s[kRadix];
  __shared__ uint32_t wcnt[kSortThreads / 32][kRadix];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) {
    const int d = threadIdx.x + j * kSortThreads;
    base_s[d] = offs[(size_t)d * ntiles + blockIdx.x];
    for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][d] = 0;
  }
  __syncthreads();
  const size_t tbase = (size_t)blockIdx.x * kSortTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i = tbase + (size_t)r * kSortThreads + threadIdx.x;
    const bool valid = i < n;
    uint64_t k = 0;
    V v{};
    unsigned d = kRadix;  // sentinel bucket for invalid lanes
    if (valid) {
      k = keys[i];
      v = vals[i];
      d = (unsigned)((k >> shift) & (kRadix - 1));
    }
    const unsigned peers = __match_any_sync(kFull, d);
    const unsigned rank = __popc(peers & lt_mask);
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t off = base_s[d] + rank;
      for (int w = 0; w < warp; ++w) off += wcnt[w][d];
      if (off < n) {  // always true for a consistent histogram
        okeys[off] = k;
        ovals[off] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kPerThread; ++j) {
      const int b = threadIdx.x + j * kSortThreads;
      uint32_t tot = 0;
      for (int w = 0; w < kSortThreads / 32; ++w) {
        tot += wcnt[w][b];
        wcnt[w][b] = 0;
      }
      base_s[b] += tot;
    }
    __syncthreads();
  }
}

template <typename V>
void radix_sort(uint64_t* keys, V* vals, uint64_t* keys_tmp, V* vals_tmp,
                size_t n, int bits, cudaStream_t s) {
  if (n <= 1 || bits <= 0) return;
  const size_t ntiles = (n + kSortTile - 1) / kSortTile;
  DevBuf<uint32_t> hist(ntiles * kRadix, s);
  uint64_t *ki = keys, *ko = keys_tmp;
  V *vi = vals, *vo = vals_tmp;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += kRadixBits, ++passes) {
    BA_LAUNCH(radix_hist_kernel<<<(unsigned)ntiles, kSortThreads, 0, s>>>(ki, n, shift, hist,
                                                                      ntiles));
    scan_rec(hist, hist, ntiles * kRadix, s);
    BA_LAUNCH((radix_scatter_kernel<V><<<(unsigned)ntiles, kSortThreads, 0, s>>>(
        ki, vi, ko, vo, n, shift, hist, ntiles)));
    std::swap(ki, ko);
    std::swap(vi, vo);
  }
  if (passes & 1) {
    check(cudaMemcpyAsync(keys, ki, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s),
          "sort copy");
    check(cudaMemcpyAsync(vals, vi, n * sizeof(V), cudaMemcpyDeviceToDevice, s), "sort copy");
  }
}

template <typename K>
__global__ void lower_bounds_kernel(const K* sorted, size_t n, uint32_t* p,
                                    size_t m, uint64_t mul) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > m) return;
  const uint64_t key = (uint64_t)i * mul;
  size_t lo = 0, hi = n;
  while (lo < hi) {
    const size_t mid = (lo + hi) >> 1;
    if ((uint64_t)sorted[mid] < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  p[i] = (uint32_t)lo;
}

}  // namespace

uint64_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n,
                            cudaStream_t s) {
  if (n == 0) return 0;
  uint32_t last_in = 0, last_out = 0;
  check(cudaMemcpyAsync(&last_in, in + n - 1, 4, cudaMemcpyDeviceToHost, s), "scan");
  scan_rec(in, out, n, s);
  check(cudaMemcpyAsync(&last_out, out + n - 1, 4, cudaMemcpyDeviceToHost, s), "scan");
  check(cudaStreamSynchronize(s), "scan sync");
  return (uint64_t)last_out + last_in;
}

void radix_sort_u64_u32(uint64_t* keys, uint32_t* vals, uint64_t* kt,
                        uint32_t* vt, size_t n, int bits, cudaStream_t s) {
  radix_sort<uint32_t>(keys, vals, kt, vt, n, bits, s);
}
void radix_sort_u64_u64(uint64_t* keys, uint64_t* vals, uint64_t* kt,
                        uint64_t* vt, size_t n, int bits, cudaStream_t s) {
  radix_sort<uint64_t>(keys, vals, kt, vt, n, bits, s);
}

void lower_bounds_u32(const uint32_t* sorted, size_t n, uint32_t* p, size_t m,
                      cudaStream_t s) {
  BA_LAUNCH(lower_bounds_kernel<uint32_t><<<grid_for(m + 1, 256), 256, 0, s>>>(sorted, n, p,
                                                                          m, 1));
}
void lower_bounds_u64(const uint64_t* sorted, size_t n, uint32_t* p, size_t m,
                      uint64_t key_mul, cudaStream_t s) {
  BA_LAUNCH(lower_bounds_kernel<uint64_t><<<grid_for(m + 1, 256), 256, 0, s>>>(sorted, n, p,
                                                                          m, key_mul));
}

}  // namespace ba
