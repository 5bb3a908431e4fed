// Stable LSD radix sort of 32-bit cell keys with a 32-bit particle-index
// payload, and the cell start table derived from the sorted keys.  Every
// kernel takes an optional device gate: when it points to 0 the kernel
// returns at once (the Verlet path keeps its rebuild in a captured step and
// runs it only on the evaluations that need one).
//
// This replaces the reference's serial linked-list rebuild
// (`linked_list_[pre_linked_list_[i]].push_back(i)` for i = 0..N-1,
// ChimeraSystem.cpp:335-338): sorting the keys stably from index order keeps
// every cell's members in ascending index order, which is the reference's
// visiting order inside a cell.
//
// Digit width is 11 bits when every key fits one digit (up to 2048 cells, one
// pass) and 8 bits otherwise.  Per pass: (1) per-tile digit histograms (the
// first pass's histogram is fused into the stage kernel), (2) one exclusive
// scan over the digit-major histogram table, (3) a stable scatter where each
// warp ranks its keys with __match_any_sync in element order and warps are
// ordered by a per-digit prefix in shared memory.
#pragma once

#include "spc_device.cuh"

namespace spc {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / kWarp;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // keys per tile
constexpr int kScanThreads = 1024;

// Tile-major digit histogram of keys[tile*2048 ...] for the digit at `shift`.
__global__ void __launch_bounds__(kSortThreads)
    k_radix_hist(const uint32_t *__restrict__ keys, int n, int shift, int bits,
                 uint32_t *__restrict__ hist, const int *gate) {
  if (gate && *gate == 0) return;
  __shared__ uint32_t h[1 << 11];
  const int R = 1 << bits;
  for (int d = threadIdx.x; d < R; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  for (int k = threadIdx.x; k < kSortTile; k += blockDim.x) {
    const int idx = base + k;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & (R - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < R; d += blockDim.x) hist[(size_t)blockIdx.x * R + d] = h[d];
}

// For many tiles the scan runs in three steps over groups of kScanGroup tiles
// (below); the register path of k_scan_digits takes at most kScanGroup tiles.
constexpr int kScanGroup = 32;

// Block-wide exclusive scan of one value per thread (kScanThreads threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t mine, uint32_t *wsum) {
  const int t = threadIdx.x, lane = t % kWarp, w = t / kWarp;
  uint32_t incl = mine;
#pragma unroll
  for (int off = 1; off < kWarp; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == kWarp - 1) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const uint32_t s = wsum[lane];
    uint32_t si = s;
#pragma unroll
    for (int off = 1; off < kWarp; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, si, off);
      if (lane >= off) si += y;
    }
    wsum[lane] = si - s;
  }
  __syncthreads();
  return wsum[w] + (incl - mine);
}

// In-place exclusive scan of the tile-major table hist[tile][digit] in
// digit-major order (all tiles of digit 0, then of digit 1, ...), which gives
// each (tile, digit) its first output position.  One block of 1024 threads.
// Up to 1024 digits and kScanGroup tiles each thread owns one digit: it loads
// the digit's counts of every tile at once (coalesced across threads, all in
// flight), keeps them in registers, and writes the running prefixes back
// after the block scan of the digit totals.  Otherwise (2048 digits, or the
// sums of more than kScanGroup groups) each thread owns two consecutive
// digits and reads their counts twice, eight loads in flight.
__global__ void __launch_bounds__(kScanThreads)
    k_scan_digits(uint32_t *__restrict__ hist, int ntiles, int bits, const int *gate) {
  if (gate && *gate == 0) return;
  __shared__ uint32_t wsum[kScanThreads / kWarp];
  const int R = 1 << bits;
  const int t = threadIdx.x;
  if (R <= kScanThreads && ntiles <= kScanGroup) {
    const bool own = t < R;
    uint32_t v[kScanGroup];
    uint32_t mine = 0;
#pragma unroll
    for (int tile = 0; tile < kScanGroup; ++tile)
      v[tile] = (own && tile < ntiles) ? hist[(size_t)tile * R + t] : 0u;
#pragma unroll
    for (int tile = 0; tile < kScanGroup; ++tile) mine += v[tile];
    uint32_t run = block_exclusive_scan(mine, wsum);
#pragma unroll
    for (int tile = 0; tile < kScanGroup; ++tile) {
      if (own && tile < ntiles) {
        hist[(size_t)tile * R + t] = run;
        run += v[tile];
      }
    }
    return;
  }
  constexpr int kPer = 2;  // up to 2048 digits
  uint32_t tot[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int d = t * kPer + k;
    uint32_t s = 0;
    if (d < R) {
      // eight independent loads in flight per iteration
      int tile = 0;
      for (; tile + 8 <= ntiles; tile += 8) {
        uint32_t v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = hist[(size_t)(tile + u) * R + d];
#pragma unroll
        for (int u = 0; u < 8; ++u) s += v[u];
      }
      for (; tile < ntiles; ++tile) s += hist[(size_t)tile * R + d];
    }
    tot[k] = s;
  }
  const uint32_t mine = tot[0] + tot[1];
  uint32_t run = block_exclusive_scan(mine, wsum);
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int d = t * kPer + k;
    if (d < R) {
      int tile = 0;
      for (; tile + 8 <= ntiles; tile += 8) {
        uint32_t v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = hist[(size_t)(tile + u) * R + d];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          hist[(size_t)(tile + u) * R + d] = run;
          run += v[u];
        }
      }
      for (; tile < ntiles; ++tile) {
        const size_t at = (size_t)tile * R + d;
        const uint32_t v = hist[at];
        hist[at] = run;
        run += v;
      }
    }
  }
}

// For many tiles the scan runs in three steps over groups of kScanGroup tiles:
// per-(group, digit) sums, a one-block digit-major scan of those sums (the
// same k_scan_digits with groups in place of tiles), and per-(group, digit)
// running prefixes written back over the group's tiles.
__global__ void k_scan_group_sums(const uint32_t *__restrict__ hist, int ntiles, int bits,
                                  uint32_t *__restrict__ part, const int *gate) {
  if (gate && *gate == 0) return;
  const int R = 1 << bits;
  const int d = blockIdx.y * blockDim.x + threadIdx.x, g = blockIdx.x;
  if (d >= R) return;
  const int t0 = g * kScanGroup, t1 = min(t0 + kScanGroup, ntiles);
  uint32_t s = 0;
  for (int t = t0; t < t1; ++t) s += hist[(size_t)t * R + d];
  part[(size_t)g * R + d] = s;
}

__global__ void k_scan_group_apply(uint32_t *__restrict__ hist, int ntiles, int bits,
                                   const uint32_t *__restrict__ part, const int *gate) {
  if (gate && *gate == 0) return;
  const int R = 1 << bits;
  const int d = blockIdx.y * blockDim.x + threadIdx.x, g = blockIdx.x;
  if (d >= R) return;
  const int t0 = g * kScanGroup, t1 = min(t0 + kScanGroup, ntiles);
  uint32_t run = part[(size_t)g * R + d];
  for (int t = t0; t < t1; ++t) {
    const size_t at = (size_t)t * R + d;
    const uint32_t v = hist[at];
    hist[at] = run;
    run += v;
  }
}

// Stable scatter of one digit pass; hist_scanned is the output of k_scan_digits.
// Each sort tile (kSortTile keys, one row of the digit table) is scattered by
// SUB CTAs of kSortTile / SUB keys, so that a small system still fills the
// GPU (SUB = 4 below kScatterSplitBelow tiles, else 1): a CTA starts from its
// tile's digit bases, adds the digit counts of the tile's earlier parts
// (shared-memory atomics: counts do not depend on their order), and ranks its
// own keys in element order, so the scatter is stable.
constexpr int kScatterSplitBelow = 2 * 152;

template <int SUB>
__global__ void __launch_bounds__(kSortThreads)
    k_radix_scatter(const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int n,
                    int shift, int bits, const uint32_t *__restrict__ hist_scanned, const int *gate) {
  constexpr int kScatterKeys = kSortTile / SUB;
  constexpr int kScatterItems = kScatterKeys / kSortThreads;
  static_assert(kScatterItems * kSortThreads * SUB == kSortTile, "scatter parts tile the sort tile");
  if (gate && *gate == 0) return;
  const int tile = blockIdx.x / SUB, part = blockIdx.x % SUB;
  const int t0 = tile * kSortTile, p0 = t0 + part * kScatterKeys;
  if (p0 >= n) return;  // a part past the end of the last tile
  extern __shared__ uint32_t smem_sort[];
  const int R = 1 << bits;
  uint32_t *wcount = smem_sort;                         // [kSortWarps][R]
  uint32_t *digit_base = smem_sort + kSortWarps * R;    // first output slot of each digit
  const int warp = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  for (int d = threadIdx.x; d < kSortWarps * R; d += blockDim.x) smem_sort[d] = 0;
  for (int d = threadIdx.x; d < R; d += blockDim.x) digit_base[d] = hist_scanned[(size_t)tile * R + d];
  __syncthreads();
  for (int idx = t0 + threadIdx.x; idx < p0; idx += blockDim.x)  // the tile's earlier parts
    atomicAdd(&digit_base[(keys_in[idx] >> shift) & (R - 1)], 1u);
  __syncthreads();

  const int base = p0 + warp * (kScatterItems * kWarp);
  const unsigned lanes_below = (1u << lane) - 1u;
  uint32_t key[kScatterItems], val[kScatterItems], rank[kScatterItems];
#pragma unroll
  for (int it = 0; it < kScatterItems; ++it) {
    const int idx = base + it * kWarp + lane;
    const bool valid = idx < n;
    key[it] = valid ? keys_in[idx] : 0u;
    val[it] = valid ? vals_in[idx] : 0u;
    // invalid lanes get a digit no valid key has, so they never share a group
    const uint32_t d = valid ? ((key[it] >> shift) & (R - 1)) : (uint32_t)R;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t r = 0xffffffffu;
    if (valid) r = wcount[warp * R + d] + __popc(peers & lanes_below);
    __syncwarp();
    if (valid && (31 - __clz(peers)) == lane) wcount[warp * R + d] += __popc(peers);
    __syncwarp();
    rank[it] = r;
  }
  __syncthreads();
  // warps are consecutive runs of elements: order them per digit
  for (int d = threadIdx.x; d < R; d += blockDim.x) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = wcount[w * R + d];
      wcount[w * R + d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kScatterItems; ++it) {
    if (rank[it] == 0xffffffffu) continue;
    const uint32_t d = (key[it] >> shift) & (R - 1);
    const uint32_t pos = digit_base[d] + wcount[warp * R + d] + rank[it];
    keys_out[pos] = key[it];
    vals_out[pos] = val[it];
  }
}

inline size_t scatter_smem_bytes(int bits) {
  return (size_t)(kSortWarps + 1) * (1u << bits) * sizeof(uint32_t);
}

// cell_start[c] = first sorted position with key >= c, for c in [0, ncell];
// every entry is written exactly once.
__device__ __forceinline__ void cell_bounds_at(const uint32_t *__restrict__ skeys, int n, int ncell,
                                               int *__restrict__ cell_start, int p) {
  const int lo = (p == 0) ? -1 : (int)skeys[p - 1];
  const int hi = (p == n) ? ncell : min((int)skeys[p], ncell);
  for (int c = lo + 1; c <= hi; ++c) cell_start[c] = p;
}

// The same for sub-cell keys 2c + h (h = 1: the upper half of cell c):
// cell_start[c] = first sorted position with key >= 2c, cell_mid[c] = first
// with key >= 2c + 1, for c in [0, ncell] and [0, ncell).  Every entry is
// written exactly once.
__device__ __forceinline__ void half_bounds_at(const uint32_t *__restrict__ skeys, int n, int ncell,
                                               int *__restrict__ cell_start, int *__restrict__ cell_mid,
                                               int p) {
  const int lo = (p == 0) ? -1 : (int)skeys[p - 1];
  const int hi = (p == n) ? 2 * ncell : min((int)skeys[p], 2 * ncell);
  for (int k = lo + 1; k <= hi; ++k) {
    if (k & 1)
      cell_mid[k >> 1] = p;
    else
      cell_start[k >> 1] = p;
  }
}

}  // namespace spc
