// Stable LSD radix sort of 32-bit cell keys with a 32-bit particle-index
// payload, and the cell start table derived from the sorted keys.
//
// This replaces the reference's serial linked-list rebuild
// (`linked_list_[pre_linked_list_[i]].push_back(i)` for i = 0..N-1,
// ChimeraSystem.cpp:335-338): sorting the keys stably from index order keeps
// every cell's members in ascending index order, which is the reference's
// visiting order inside a cell.
//
// Per 8-bit digit pass: (1) per-tile digit histograms, (2) one exclusive scan
// over the digit-major histogram table, (3) a stable scatter where each warp
// ranks its keys with __match_any_sync in element order and warps are ordered
// by a per-digit prefix in shared memory.
#pragma once

#include "spc_device.cuh"

namespace spc {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / kWarp;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // keys per tile
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kScanThreads = 1024;

__global__ void __launch_bounds__(kSortThreads)
    k_radix_hist(const uint32_t *__restrict__ keys, int n, int shift, int ntiles,
                 uint32_t *__restrict__ hist) {
  __shared__ uint32_t h[kRadix];
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  for (int k = threadIdx.x; k < kSortTile; k += blockDim.x) {
    const int idx = base + k;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) hist[(size_t)d * ntiles + blockIdx.x] = h[d];
}

// Exclusive scan of data[0..m) in place, one block of kScanThreads threads.
__global__ void __launch_bounds__(kScanThreads) k_scan_exclusive(uint32_t *__restrict__ data, int m) {
  __shared__ uint32_t sums[kScanThreads];
  const int t = threadIdx.x;
  const int per = (m + kScanThreads - 1) / kScanThreads;
  const int a = min(t * per, m), b = min(a + per, m);
  uint32_t s = 0;
  for (int i = a; i < b; ++i) s += data[i];
  sums[t] = s;
  __syncthreads();
  for (int off = 1; off < kScanThreads; off <<= 1) {
    const uint32_t v = t >= off ? sums[t - off] : 0u;
    __syncthreads();
    sums[t] += v;
    __syncthreads();
  }
  uint32_t run = t ? sums[t - 1] : 0u;
  for (int i = a; i < b; ++i) {
    const uint32_t v = data[i];
    data[i] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(kSortThreads)
    k_radix_scatter(const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int n,
                    int shift, int ntiles, const uint32_t *__restrict__ hist_scanned) {
  __shared__ uint32_t wcount[kSortWarps][kRadix];
  __shared__ uint32_t tile_base_of_digit[kRadix];
  const int warp = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  for (int d = threadIdx.x; d < kSortWarps * kRadix; d += blockDim.x) (&wcount[0][0])[d] = 0;
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
    tile_base_of_digit[d] = hist_scanned[(size_t)d * ntiles + blockIdx.x];
  __syncthreads();

  const int base = blockIdx.x * kSortTile + warp * (kSortItems * kWarp);
  const unsigned lanes_below = (1u << lane) - 1u;
  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    const int idx = base + it * kWarp + lane;
    const bool valid = idx < n;
    key[it] = valid ? keys_in[idx] : 0u;
    val[it] = valid ? vals_in[idx] : 0u;
    // invalid lanes get a digit no valid key has, so they never share a group
    const uint32_t d = valid ? ((key[it] >> shift) & (kRadix - 1)) : (uint32_t)kRadix;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t r = 0xffffffffu;
    if (valid) r = wcount[warp][d] + __popc(peers & lanes_below);
    __syncwarp();
    if (valid && (31 - __clz(peers)) == lane) wcount[warp][d] += __popc(peers);
    __syncwarp();
    rank[it] = r;
  }
  __syncthreads();
  // warps are consecutive runs of elements: order them per digit
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = wcount[w][d];
      wcount[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    if (rank[it] == 0xffffffffu) continue;
    const uint32_t d = (key[it] >> shift) & (kRadix - 1);
    const uint32_t pos = tile_base_of_digit[d] + wcount[warp][d] + rank[it];
    keys_out[pos] = key[it];
    vals_out[pos] = val[it];
  }
}

// cell_start[c] = first sorted position with key >= c, for c in [0, ncell];
// every entry is written exactly once.
__global__ void k_cell_bounds(const uint32_t *__restrict__ skeys, int n, int ncell,
                              int *__restrict__ cell_start) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > n) return;
  const int lo = (p == 0) ? -1 : (int)skeys[p - 1];
  const int hi = (p == n) ? ncell : min((int)skeys[p], ncell);
  for (int c = lo + 1; c <= hi; ++c) cell_start[c] = p;
}

}  // namespace spc
