// Cell-tile neighbour passes: one CTA per cell.
//
// The CTA stages the candidates of the cell's 3x3 stencil (in the reference's
// visiting order, ChimeraSystem.cpp:39-44; ascending index inside a cell) into
// shared memory once, with each stencil cell's periodic shift already added to
// the float prefilter coordinates, and then every thread of the CTA works on
// one particle of the cell against that list: no global load in the inner
// loop, and every candidate read is a shared-memory broadcast.
//
// FP32C (k_tile_fp32c): the candidate list is split among up to four warps per
// 32-particle chunk to keep ~27 warps resident per SM; each part sums blocks of
// 32 terms in float and adds each block sum with Kahan compensation; the parts
// are combined in a fixed order, so results are deterministic.
//
// FP64 (k_tile_fp64): one thread per particle walks the whole list in order,
// so each particle's sum keeps the reference's order term for term.  Accepted
// candidates go into a per-thread FIFO in shared memory and the warp drains
// the common minimum of its queues after every block of 32 candidates, so the
// FP64 sin/cos (1/64-rate pipe on GB300) runs on full warps instead of on the
// few lanes that happen to accept a given candidate.
//
// Both decide every pair exactly as the reference: float prefilter on
// cell-relative coordinates, the reference's FP64 test for pairs within a
// relative 3e-5 of rho^2 (warp-uniform branch, rare).
#pragma once

#include "spc_kernels.cuh"

namespace spc {

constexpr int kTileCap = 1024;      // FP32C: candidates staged per round
constexpr int kTileCap64 = 768;     // FP64: candidates staged per round (7 CTAs/SM fit)
constexpr int kTileThreads32 = 128; // FP32C CTA: 4 warps
constexpr int kTileThreads64 = 64;  // FP64 CTA: 2 warps
constexpr int kQCap = 64;           // FP64 per-thread queue (power of two)

struct Stencil {
  int start[9];    // cell-order start of each stencil cell
  int prefix[10];  // offsets of each stencil cell in the staged list
};

// half < 0: the 3x3 stencil of cell c.  half 0 / 1 (sub-cells): the stencil
// of the lower / upper half of cell c.  A particle of the lower half is more
// than a cell side (>= rho) below the upper half of the row above, so that
// row's entries keep only their lower half [start, mid); the upper half's
// stencil keeps the upper half [mid, end) of the row below.  The own cell
// (entry 4) stays whole, and so does a far cell when both it and cell c hold
// a particle near the half line (cell_near, kNearHalf).
__device__ __forceinline__ void stencil_of(const KArgs &a, const SysDesc &sd, int c, Stencil &s,
                                           int half = -1) {
  const SysConst &sc = sd.sc;
  const int nc = sc.nc, cl = c - sd.c0, cx = cl % nc, cy = cl / nc;
  const bool near = half >= 0 && a.cell_near[c];
  s.prefix[0] = 0;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int ox = (q % 3) - 1, oy = (q / 3) - 1;
    const int cj = sd.c0 + adjust_cell(cy + oy, nc) * nc + adjust_cell(cx + ox, nc);
    int ja = a.cell_start[cj], jb = a.cell_start[cj + 1];
    if (half >= 0 && oy == (half == 0 ? 1 : -1) && !(near && a.cell_near[cj])) {
      if (half == 0)
        jb = a.cell_mid[cj];
      else
        ja = a.cell_mid[cj];
    }
    s.start[q] = ja;
    s.prefix[q + 1] = s.prefix[q] + (jb - ja);
  }
}

// Cell-order slot of staged candidate g (0 <= g < prefix[9]) and its stencil
// entry q.  A select chain with constant indices keeps the stencil in
// registers (a dynamic index would put it in local memory).
__device__ __forceinline__ int slot_of(const Stencil &s, int g, int &q_out) {
  int q = 0, base = s.start[0];
#pragma unroll
  for (int k = 1; k < 9; ++k) {
    const bool ge = g >= s.prefix[k];
    q = ge ? k : q;
    base = ge ? s.start[k] - s.prefix[k] : base;
  }
  q_out = q;
  return base + g;
}

// periodic shift of stencil entry q in the float prefilter frame
__device__ __forceinline__ float shift_x(int q, float cell_f) { return (float)(q % 3 - 1) * cell_f; }
__device__ __forceinline__ float shift_y(int q, float cell_f) { return (float)(q / 3 - 1) * cell_f; }

// ---------------------------------------------------------------------------
// FP32C passes.  Pass 1 (KIND == kKindSin) also records, for cells whose
// candidate list fits one staging round, each particle's neighbour set as a
// bitmask over that list; pass 2 (kKindCos2) then walks only the set bits
// instead of re-testing every candidate.  Cells with more candidates run the
// filter in pass 2 as well.  The masks are laid out by mask_at, so pass 2
// fetches the words of four candidate blocks with one 16-byte load.
constexpr int kMaskWords = kTileCap / 32;
static_assert(kMaskWords % 4 == 0, "mask words come in groups of four");

// Work item `item` of the cell-tile kernels: cell c = item / K and part
// item % K of its particles, K = a.tile_split CTAs per cell.  A part is a
// whole number of the kernel's particle groups (GROUP = the CTA's threads,
// the particles it processes at a time), so a cell of at most GROUP
// particles stays one item and is staged once, while the few cells of a
// clustered state that hold several groups are spread over up to K CTAs
// instead of running their groups one after another on one CTA (the tail of
// a single-wave pass).  Items past a cell's last group are empty.  c0 is the
// cell's first particle (the own cell's stencil entry starts there).
struct TileItem {
  int c, c0, cb, ce;
};

__device__ __forceinline__ int tile_items(const KArgs &a) { return a.ncell_tile * max(a.tile_split, 1); }

template <int GROUP>
__device__ __forceinline__ bool tile_item(const KArgs &a, int item, TileItem &t) {
  const int K = max(a.tile_split, 1);
  t.c = item / K;
  const int h = item - t.c * K;
  t.c0 = a.cell_start[t.c];
  const int c1 = a.cell_start[t.c + 1];
  const int groups = (c1 - t.c0 + GROUP - 1) / GROUP;
  const int per = ((groups + K - 1) / K) * GROUP;
  t.cb = t.c0 + h * per;
  t.ce = min(c1, t.cb + per);
  return t.cb < t.ce;
}

// Per-part results of one 128-particle group: each part's compensated sums
// (sum minus compensation) and counts; pass 1 has one sum, pass 2 two.
template <int KIND>
struct TileRed {
  float s0[4][kTileThreads32];
  float s1[KIND == kKindCos2 ? 4 : 1][kTileThreads32];
  int n[4][kTileThreads32];
};

// Shared memory of k_tile_fp32c is kept under ~31 KB (and registers at 72)
// so that 7 CTAs fit an SM: a 1024-cell system then runs in a single wave.
constexpr int kTileMinBlocks32 = 7;

__device__ __forceinline__ int split_point(int rcnt, int part, int S) {
  // part boundaries on multiples of 32 so that mask words are not shared
  return part >= S ? rcnt : ((rcnt * part / S) & ~31);
}

// One block of 32 staged candidates against one particle (FP32C).  The block
// is fully unrolled: bit t of *bits is candidate j0 + t.  SELF: the block may
// contain the particle itself (staged index `self`).  Pairs the float test
// cannot decide are left out here and reported through *mn (the smallest
// |d^2 - mid| seen).  The block sums the inside candidates' cos phi_j and
// sin phi_j (and, pass 2, the same weighted by the phase rate d_j); the
// caller turns them into the alignment terms by angle addition once per block.
template <int KIND, bool SELF>
__device__ __forceinline__ void block32(const float4 *__restrict__ s_c4, const float *__restrict__ s_d,
                                        int j0, int self, float fxi, float fyi, float nmid, float nband,
                                        float &sc_, float &ss_, float &sdc, float &sds, uint32_t &bits,
                                        float &mn) {
#pragma unroll
  for (int t = 0; t < kWarp; ++t) {
    const float4 cj = s_c4[j0 + t];
    const float dx = cj.x - fxi, dy = cj.y - fyi;
    float off = cutoff_offset(dx, dy, nmid);
    bool in = off < nband;
    if (SELF) {
      in = in && (j0 + t != self);
      off = (j0 + t != self) ? off : 3.0e38f;
    }
    mn = fminf(mn, fabsf(off));
    addf2_if(sc_, ss_, cj.z, cj.w, in);
    if constexpr (KIND == kKindCos2) fmaf2_if(sdc, sds, s_d[j0 + t], cj.z, cj.w, in);
    bits |= (uint32_t)in << t;
  }
}

// Stage candidates [rlo, rlo + rcnt) of the stencil list (padded to rpad) for
// the FP32C passes.  This and part_fp32c serve the units kernel; the cell-tile
// kernel keeps the same code inline, as it was before the units existed (a
// version of it that called these helpers compiled to more spills and ran
// pass 1 slower).
template <int KIND>
__device__ __forceinline__ void stage_fp32c(const KArgs &a, const SysConst &sc, const Stencil &st, int rlo,
                                            int rcnt, int rpad, float4 *s_c4, float *s_d) {
  for (int k = threadIdx.x; k < rpad; k += blockDim.x) {
    if (k < rcnt) {
      int q;
      const int pj = slot_of(st, rlo + k, q);
      const float2 f = a.fxy[pj];
      const float2 cs = a.cs[pj];
      s_c4[k] = make_float4(f.x + shift_x(q, sc.cell_f), f.y + shift_y(q, sc.cell_f), cs.x, cs.y);
      if constexpr (KIND == kKindCos2) s_d[k] = a.dphi_f[pj];
    } else {  // padding: far away, never a neighbour, never near the cutoff
      s_c4[k] = make_float4(3.0e18f, 3.0e18f, 0.0f, 0.0f);
      if constexpr (KIND == kKindCos2) s_d[k] = 0.0f;
    }
  }
}

// One warp: particle ig + li of a group of gi (lane li; li >= gi idle) against
// part [jlo, jhi) of the staged round [rlo, rlo + rcnt); its compensated sums
// and count go to red.*[part][li].  Called by all 32 lanes of the warp.
template <int KIND>
__device__ __forceinline__ void part_fp32c(const KArgs &a, const SysConst &sc, const Stencil &st,
                                           const float4 *s_c4, const float *s_d, TileRed<KIND> &red,
                                           int c0, int ig, int li, int gi, int rlo, int rcnt, int jlo,
                                           int jhi, int part, bool masked, bool exact_all, float band,
                                           float nmid) {
  const int n_all = a.n_active;
  const bool valid = li < gi;
  const int p = ig + li;
  float fxi = 3.0e30f, fyi = 3.0e30f, ca = 0.0f, sa = 0.0f, di = 0.0f;
  double xi = 0.0, yi = 0.0;
  if (valid) {
    const float2 f = a.fxy[p];
    fxi = f.x;
    fyi = f.y;
    const float2 t = a.cs[p];  // cos / sin of phi_i + alpha by angle addition
    ca = t.x * sc.cos_a - t.y * sc.sin_a;
    sa = t.y * sc.cos_a + t.x * sc.sin_a;
    if constexpr (KIND == kKindCos2) di = a.dphi_f[p];
    xi = a.sx[p];
    yi = a.sy[p];
  }
  // staged index of i itself (the own cell is stencil entry 4); its block
  const int self = st.prefix[4] + (p - c0) - rlo;
  float S0 = 0.0f, C0 = 0.0f, S1 = 0.0f, C1 = 0.0f;
  int n = 0;
  if (KIND == kKindCos2 && masked) {
    // pass 2 over the neighbour bitmask of pass 1 (same staged list):
    // one 16-byte group of four mask words in hand, the next in flight
    const uint4 *m4 = reinterpret_cast<const uint4 *>(a.nbmask);
    const uint4 none = make_uint4(0u, 0u, 0u, 0u);
    const int w0 = jlo / kWarp, w1 = jhi / kWarp;
    int g = w0 >> 2;
    uint4 cur = (valid && w0 < w1) ? m4[(size_t)g * n_all + p] : none;
    uint4 nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
    for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
      const int w = j0 / kWarp;
      if ((w >> 2) != g) {
        ++g;
        cur = nxt;
        nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
      }
      const int sub = w & 3;
      const uint32_t bits = sub == 0 ? cur.x : sub == 1 ? cur.y : sub == 2 ? cur.z : cur.w;
      float sc_ = 0.0f, ss_ = 0.0f, sdc = 0.0f, sds = 0.0f;
#pragma unroll
      for (int t = 0; t < kWarp; ++t) {
        if ((bits >> t) & 1u) {
          const float4 cj = s_c4[j0 + t];
          const float dj = s_d[j0 + t];
          sc_ += cj.z;
          ss_ += cj.w;
          sdc = fmaf(dj, cj.z, sdc);
          sds = fmaf(dj, cj.w, sds);
        }
      }
      // sum cos(phi_j - phi_i - alpha) and sum (d_j - d_i) cos(...)
      const float b0 = fmaf(sc_, ca, ss_ * sa);
      const float b1 = fmaf(sdc, ca, fmaf(sds, sa, -di * b0));
      n += __popc(bits);
      kahan_add(S0, C0, b0);
      kahan_add(S1, C1, b1);
    }
  } else {
    for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
      float sc_ = 0.0f, ss_ = 0.0f, sdc = 0.0f, sds = 0.0f, mn = 3.0e38f;
      uint32_t bits = 0u;
      const bool self_block = (unsigned)(self - j0) < (unsigned)kWarp;
      if (!exact_all) {
        if (__any_sync(0xffffffffu, self_block))
          block32<KIND, true>(s_c4, s_d, j0, self, fxi, fyi, nmid, -band, sc_, ss_, sdc, sds, bits, mn);
        else
          block32<KIND, false>(s_c4, s_d, j0, self, fxi, fyi, nmid, -band, sc_, ss_, sdc, sds, bits, mn);
      }
      // the block's alignment terms by angle addition:
      // sin(phi_j - phi_i - alpha) = sin phi_j ca - cos phi_j sa,
      // cos(phi_j - phi_i - alpha) = cos phi_j ca + sin phi_j sa
      float b0, b1 = 0.0f;
      if constexpr (KIND == kKindSin) {
        b0 = fmaf(ss_, ca, -sc_ * sa);
      } else {
        b0 = fmaf(sc_, ca, ss_ * sa);
        b1 = fmaf(sdc, ca, fmaf(sds, sa, -di * b0));
      }
      // pairs the float test cannot decide: the reference's FP64 test
      const bool amb = valid && (exact_all || mn <= band);
      if (__any_sync(0xffffffffu, amb)) {
        if (amb) {
          for (int t = 0; t < kWarp; ++t) {
            const int j = j0 + t;
            if (j == self || j >= rcnt) continue;
            const float4 cj = s_c4[j];
            const float dx = cj.x - fxi, dy = cj.y - fyi;
            if (!(exact_all || fabsf(cutoff_offset(dx, dy, nmid)) <= band)) continue;
            int q;
            const int pj = slot_of(st, rlo + j, q);
            if (!exact_within(sc, xi, yi, a.sx[pj], a.sy[pj])) continue;
            if constexpr (KIND == kKindSin) {
              b0 += fmaf(cj.w, ca, -cj.z * sa);
            } else {
              const float tv = fmaf(cj.z, ca, cj.w * sa);
              b0 += tv;
              b1 = fmaf(s_d[j] - di, tv, b1);
            }
            bits |= 1u << t;
          }
        }
      }
      n += __popc(bits);
      kahan_add(S0, C0, b0);
      if constexpr (KIND == kKindCos2) kahan_add(S1, C1, b1);
      if (KIND == kKindSin && masked && valid) a.nbmask[mask_at(j0 / kWarp, p, n_all)] = bits;
    }
  }
  if (valid) {
    red.s0[part][li] = S0 - C0;
    if constexpr (KIND == kKindCos2) red.s1[part][li] = S1 - C1;
    red.n[part][li] = n;
  }
}

// Parts 0..S-1 of thread tid's particle added, in order, to a running
// compensated sum.
template <int KIND>
__device__ __forceinline__ void add_parts(const TileRed<KIND> &red, int S, int tid, float &ts, float &tc,
                                          float &ts1, float &tc1, int &tn) {
  for (int part = 0; part < S; ++part) {
    kahan_add(ts, tc, red.s0[part][tid]);
    tn += red.n[part][tid];
  }
  if constexpr (KIND == kKindCos2)
    for (int part = 0; part < S; ++part) kahan_add(ts1, tc1, red.s1[part][tid]);
}

template <int KIND>
__device__ __forceinline__ void finish_fp32c(const KArgs &a, int epi, const SysDesc &sd, int p, float s0,
                                             float s1, int n) {
  ILane il;
  load_i<kPrecFP32C, KIND>(a, sd.sc, il, p, true);
  Acc<kPrecFP32C> acc;
  acc.init();
  acc.s0 = s0;
  if constexpr (KIND == kKindCos2) acc.s1 = s1;
  acc.n = n;
  epilogue<kPrecFP32C, KIND>(a, epi, sd, il, acc, a.pidx[p]);
}

// Cell units (tuning SPC_TUNE_CELL_UNITS).  Every cell whose candidate list
// takes at most kSplitRounds staging rounds is cut into units of 32 particles
// x one staging round, and the units kernel runs each unit on its own CTA,
// beside the cell-tile kernel, which keeps only the cells of longer lists.
// On a clustered state the cell-tile kernel's one CTA per 128-particle group
// is badly balanced: a cell of a cluster holds up to ~380 particles with
// ~6,000 candidates, several times a typical cell's work, and its groups set
// the end of the single-wave pass while most SMs idle.  Units of ~32 x 1,024
// pair tests spread that work over every SM.  A unit's four warps take a
// quarter of its round each; the unit stores its per-particle sums of the
// round, and the last unit of a 32-particle chunk to finish (a counter per
// chunk, reset by that unit) adds the rounds in order and finishes the
// particles.  k_list_units lists the units once per evaluation (both passes
// see the same cells).  Which cells are units, and the order of every sum,
// depend on the cell alone, so the results do not depend on the CTAs per cell.
// With sub-cells (SPC_TUNE_SUBCELLS, cell_mid set) each half of a unit cell
// is cut the same way over its own half stencil (stencil_of with half 0 / 1)
// and listed as (2c + half, u); the cell stays a unit cell on its whole
// stencil's round count, which bounds both halves'.
constexpr int kSplitRounds = 8;

__device__ __forceinline__ bool unit_cell(const KArgs &a, int n_c, int total, int cap) {
  return a.units != nullptr && n_c > 0 && total <= kSplitRounds * cap;
}

// List the units of every unit cell of the cell-tile systems (one thread per
// cell), once per evaluation after the gather, for both passes' units kernels,
// and mark those cells for the cell-tile kernels to skip.
// CAP: the form's staging round.
template <int CAP>
__global__ void k_list_units(KArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.ncell_tile) return;
  const int c0 = a.cell_start[c], n_c = a.cell_start[c + 1] - c0;
  a.cell_unit[c] = 0;
  if (n_c == 0) return;
  const SysDesc &sd = a.sys[a.sys_of_c[c]];
  if (sd.sc.allpairs) return;
  Stencil st;
  stencil_of(a, sd, c, st);
  const int total = st.prefix[9];
  if (!unit_cell(a, n_c, total, CAP)) return;
  a.cell_unit[c] = 1;
  if (a.cell_mid) {
    // sub-cells: each half's units over its own stencil, listed as (2c + half, u)
    const int mid = a.cell_mid[c];
    for (int h = 0; h < 2; ++h) {
      const int n_h = h ? c0 + n_c - mid : mid - c0;
      if (n_h == 0) continue;
      Stencil sh;
      stencil_of(a, sd, c, sh, h);
      const int rounds = (sh.prefix[9] + CAP - 1) / CAP;
      const int units = (n_h + kWarp - 1) / kWarp * rounds;
      const int base = atomicAdd(a.unit_count, units);
      for (int u = 0; u < units; ++u) a.units[base + u] = make_int2(2 * c + h, u);
    }
    return;
  }
  const int rounds = (total + CAP - 1) / CAP;
  const int units = (n_c + kWarp - 1) / kWarp * rounds;
  const int base = atomicAdd(a.unit_count, units);
  for (int u = 0; u < units; ++u) a.units[base + u] = make_int2(c, u);
}

// UNITS: unit cells are left to the units kernel (a separate instantiation, so
// that the kernel without cell units compiles exactly as before).
template <int KIND, bool UNITS>
__global__ void __launch_bounds__(kTileThreads32, kTileMinBlocks32) k_tile_fp32c(KArgs a, int epi) {
  __shared__ float4 s_c4[kTileCap];   // x+shift, y+shift, cos phi, sin phi (padded to 32)
  __shared__ float s_d[KIND == kKindCos2 ? kTileCap : 1];  // pass 2: phase rate (float)
  __shared__ TileRed<KIND> red;
  constexpr int kT2 = KIND == kKindCos2 ? kTileThreads32 : 1;
  __shared__ float t_s[kTileThreads32], t_c[kTileThreads32], t_s1[kT2], t_c1[kT2];
  __shared__ int t_n[kTileThreads32];
  const int n_all = a.n_active;
  const int tid = threadIdx.x, w = tid / kWarp, lane = tid % kWarp;
  const int nitems = tile_items(a);
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    TileItem ti;
    if (!tile_item<kTileThreads32>(a, item, ti)) continue;
    if constexpr (UNITS) {
      if (a.cell_unit[ti.c]) continue;  // run by the units kernel
    }
    const int c = ti.c, c0 = ti.c0, cb = ti.cb, ce = ti.ce;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    Stencil st;
    stencil_of(a, sd, c, st);
    const int total = st.prefix[9];
    const int rounds = (total + kTileCap - 1) / kTileCap;
    const bool masked = rounds == 1 && a.nbmask != nullptr && !exact_all;
    for (int ig = cb; ig < ce; ig += kTileThreads32) {
      const int gi = min(kTileThreads32, ce - ig);
      if (tid < gi) {
        t_s[tid] = t_c[tid] = 0.0f;
        if constexpr (KIND == kKindCos2) t_s1[tid] = t_c1[tid] = 0.0f;
        t_n[tid] = 0;
      }
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kTileCap, rcnt = min(kTileCap, total - rlo);
        const int rpad = (rcnt + kWarp - 1) & ~(kWarp - 1);
        if (rounds > 1 || ig == cb) {
          __syncthreads();
          for (int k = tid; k < rpad; k += blockDim.x) {
            if (k < rcnt) {
              int q;
              const int pj = slot_of(st, rlo + k, q);
              const float2 f = a.fxy[pj];
              const float2 cs = a.cs[pj];
              s_c4[k] = make_float4(f.x + shift_x(q, sc.cell_f), f.y + shift_y(q, sc.cell_f), cs.x, cs.y);
              if constexpr (KIND == kKindCos2) s_d[k] = a.dphi_f[pj];
            } else {  // padding: far away, never a neighbour, never near the cutoff
              s_c4[k] = make_float4(3.0e18f, 3.0e18f, 0.0f, 0.0f);
              if constexpr (KIND == kKindCos2) s_d[k] = 0.0f;
            }
          }
          __syncthreads();
        }
        // work items: (chunk of 32 particles, part of the candidate list)
        const int chunks = (gi + kWarp - 1) / kWarp;
        const int S = chunks >= 4 ? 1 : (chunks == 1 ? 4 : 2);
        const int items = chunks * S;
        for (int item = w; item < items; item += kTileThreads32 / kWarp) {
          const int chunk = item / S, part = item % S;
          const int li = chunk * kWarp + lane;  // particle within the group
          const bool valid = li < gi;
          const int p = ig + li;
          float fxi = 3.0e30f, fyi = 3.0e30f, ca = 0.0f, sa = 0.0f, di = 0.0f;
          double xi = 0.0, yi = 0.0;
          if (valid) {
            const float2 f = a.fxy[p];
            fxi = f.x;
            fyi = f.y;
            const float2 t = a.cs[p];  // cos / sin of phi_i + alpha by angle addition
            ca = t.x * sc.cos_a - t.y * sc.sin_a;
            sa = t.y * sc.cos_a + t.x * sc.sin_a;
            if constexpr (KIND == kKindCos2) di = a.dphi_f[p];
            xi = a.sx[p];
            yi = a.sy[p];
          }
          // staged index of i itself (the own cell is stencil entry 4); its block
          const int self = st.prefix[4] + (p - c0) - rlo;
          const int jlo = split_point(rpad, part, S), jhi = split_point(rpad, part + 1, S);
          float S0 = 0.0f, C0 = 0.0f, S1 = 0.0f, C1 = 0.0f;
          int n = 0;
          if (KIND == kKindCos2 && masked) {
            // pass 2 over the neighbour bitmask of pass 1 (same staged list):
            // one 16-byte group of four mask words in hand, the next in flight
            const uint4 *m4 = reinterpret_cast<const uint4 *>(a.nbmask);
            const uint4 none = make_uint4(0u, 0u, 0u, 0u);
            const int w0 = jlo / kWarp, w1 = jhi / kWarp;
            int g = w0 >> 2;
            uint4 cur = (valid && w0 < w1) ? m4[(size_t)g * n_all + p] : none;
            uint4 nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
            for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
              const int w = j0 / kWarp;
              if ((w >> 2) != g) {
                ++g;
                cur = nxt;
                nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
              }
              const int sub = w & 3;
              const uint32_t bits = sub == 0 ? cur.x : sub == 1 ? cur.y : sub == 2 ? cur.z : cur.w;
              float sc_ = 0.0f, ss_ = 0.0f, sdc = 0.0f, sds = 0.0f;
#pragma unroll
              for (int t = 0; t < kWarp; ++t) {
                if ((bits >> t) & 1u) {
                  const float4 cj = s_c4[j0 + t];
                  const float dj = s_d[j0 + t];
                  sc_ += cj.z;
                  ss_ += cj.w;
                  sdc = fmaf(dj, cj.z, sdc);
                  sds = fmaf(dj, cj.w, sds);
                }
              }
              // sum cos(phi_j - phi_i - alpha) and sum (d_j - d_i) cos(...)
              const float b0 = fmaf(sc_, ca, ss_ * sa);
              const float b1 = fmaf(sdc, ca, fmaf(sds, sa, -di * b0));
              n += __popc(bits);
              kahan_add(S0, C0, b0);
              kahan_add(S1, C1, b1);
            }
          } else {
            for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
              float sc_ = 0.0f, ss_ = 0.0f, sdc = 0.0f, sds = 0.0f, mn = 3.0e38f;
              uint32_t bits = 0u;
              const bool self_block = (unsigned)(self - j0) < (unsigned)kWarp;
              if (!exact_all) {
                if (__any_sync(0xffffffffu, self_block))
                  block32<KIND, true>(s_c4, s_d, j0, self, fxi, fyi, nmid, -band, sc_, ss_, sdc, sds, bits, mn);
                else
                  block32<KIND, false>(s_c4, s_d, j0, self, fxi, fyi, nmid, -band, sc_, ss_, sdc, sds, bits, mn);
              }
              // the block's alignment terms by angle addition:
              // sin(phi_j - phi_i - alpha) = sin phi_j ca - cos phi_j sa,
              // cos(phi_j - phi_i - alpha) = cos phi_j ca + sin phi_j sa
              float b0, b1 = 0.0f;
              if constexpr (KIND == kKindSin) {
                b0 = fmaf(ss_, ca, -sc_ * sa);
              } else {
                b0 = fmaf(sc_, ca, ss_ * sa);
                b1 = fmaf(sdc, ca, fmaf(sds, sa, -di * b0));
              }
              // pairs the float test cannot decide: the reference's FP64 test
              const bool amb = valid && (exact_all || mn <= band);
              if (__any_sync(0xffffffffu, amb)) {
                if (amb) {
                  for (int t = 0; t < kWarp; ++t) {
                    const int j = j0 + t;
                    if (j == self || j >= rcnt) continue;
                    const float4 cj = s_c4[j];
                    const float dx = cj.x - fxi, dy = cj.y - fyi;
                    if (!(exact_all || fabsf(cutoff_offset(dx, dy, nmid)) <= band)) continue;
                    int q;
                    const int pj = slot_of(st, rlo + j, q);
                    if (!exact_within(sc, xi, yi, a.sx[pj], a.sy[pj])) continue;
                    if constexpr (KIND == kKindSin) {
                      b0 += fmaf(cj.w, ca, -cj.z * sa);
                    } else {
                      const float tv = fmaf(cj.z, ca, cj.w * sa);
                      b0 += tv;
                      b1 = fmaf(s_d[j] - di, tv, b1);
                    }
                    bits |= 1u << t;
                  }
                }
              }
              n += __popc(bits);
              kahan_add(S0, C0, b0);
              if constexpr (KIND == kKindCos2) kahan_add(S1, C1, b1);
              if (KIND == kKindSin && masked && valid)
                a.nbmask[mask_at(j0 / kWarp, p, n_all)] = bits;
            }
          }
          if (valid) {
            red.s0[part][li] = S0 - C0;
            if constexpr (KIND == kKindCos2) red.s1[part][li] = S1 - C1;
            red.n[part][li] = n;
          }
        }
        __syncthreads();
        if (tid < gi) {
          float ts = t_s[tid], tc = t_c[tid];
          int tn = t_n[tid];
          for (int part = 0; part < S; ++part) {
            kahan_add(ts, tc, red.s0[part][tid]);
            tn += red.n[part][tid];
          }
          t_s[tid] = ts;
          t_c[tid] = tc;
          t_n[tid] = tn;
          if constexpr (KIND == kKindCos2) {
            float ts1 = t_s1[tid], tc1 = t_c1[tid];
            for (int part = 0; part < S; ++part) kahan_add(ts1, tc1, red.s1[part][tid]);
            t_s1[tid] = ts1;
            t_c1[tid] = tc1;
          }
        }
      }
      if (tid < gi) {
        const int p = ig + tid;
        ILane il;
        load_i<kPrecFP32C, KIND>(a, sc, il, p, true);
        Acc<kPrecFP32C> acc;
        acc.init();
        acc.s0 = t_s[tid] - t_c[tid];
        if constexpr (KIND == kKindCos2) acc.s1 = t_s1[tid] - t_c1[tid];
        acc.n = t_n[tid];
        epilogue<kPrecFP32C, KIND>(a, epi, sd, il, acc, a.pidx[p]);
      }
      __syncthreads();
    }
  }
}

// The units of an FP32C pass (listed by k_list_units after the gather):
// unit u of cell c is chunk u / rounds (32 particles) x staging round
// u % rounds, its list split among the four warps.
template <int KIND>
__global__ void __launch_bounds__(kTileThreads32, kTileMinBlocks32) k_units_fp32c(KArgs a, int epi) {
  __shared__ float4 s_c4[kTileCap];
  __shared__ float s_d[KIND == kKindCos2 ? kTileCap : 1];
  __shared__ TileRed<KIND> red;
  __shared__ int s_last;
  const int n_all = a.n_active;
  const int tid = threadIdx.x, w = tid / kWarp, lane = tid % kWarp;
  const int count = *a.unit_count;
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const int2 e = a.units[i];
    // the unit's cell and, with sub-cells, its half: particles [g0, g1)
    const int c = a.cell_mid ? e.x >> 1 : e.x, half = a.cell_mid ? e.x & 1 : -1;
    const int c0 = a.cell_start[c];
    const int g0 = half == 1 ? a.cell_mid[c] : c0;
    const int g1 = half == 0 ? a.cell_mid[c] : a.cell_start[c + 1];
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    Stencil st;
    stencil_of(a, sd, c, st, half);
    const int total = st.prefix[9];
    const int rounds = (total + kTileCap - 1) / kTileCap;
    const bool masked = rounds == 1 && a.nbmask != nullptr && !exact_all;
    const int k = e.y / rounds, r = e.y - k * rounds;
    const int ig = g0 + k * kWarp, gi = min(kWarp, g1 - ig);
    const int rlo = r * kTileCap, rcnt = min(kTileCap, total - rlo);
    const int rpad = (rcnt + kWarp - 1) & ~(kWarp - 1);
    __syncthreads();
    stage_fp32c<KIND>(a, sc, st, rlo, rcnt, rpad, s_c4, s_d);
    __syncthreads();
    part_fp32c<KIND>(a, sc, st, s_c4, s_d, red, c0, ig, lane, gi, rlo, rcnt, split_point(rpad, w, 4),
                     split_point(rpad, w + 1, 4), w, masked, exact_all, band, nmid);
    __syncthreads();
    float ts = 0.0f, tc = 0.0f, ts1 = 0.0f, tc1 = 0.0f;
    int tn = 0;
    if (tid < gi) add_parts<KIND>(red, 4, tid, ts, tc, ts1, tc1, tn);
    const int p = ig + tid;
    if (rounds == 1) {
      if (tid < gi) finish_fp32c<KIND>(a, epi, sd, p, ts - tc, ts1 - tc1, tn);
      continue;
    }
    if (tid < gi) {
      a.part_f[(size_t)r * n_all + p] = make_float2(ts - tc, ts1 - tc1);
      a.part_n[(size_t)r * n_all + p] = tn;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&a.unit_done[ig], 1) == rounds - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      if (tid < gi) {
        float s0 = 0.0f, cc0 = 0.0f, s1 = 0.0f, cc1 = 0.0f;
        int nn = 0;
        for (int q = 0; q < rounds; ++q) {
          const float2 v = __ldcg(&a.part_f[(size_t)q * n_all + p]);
          kahan_add(s0, cc0, v.x);
          if constexpr (KIND == kKindCos2) kahan_add(s1, cc1, v.y);
          nn += __ldcg(&a.part_n[(size_t)q * n_all + p]);
        }
        finish_fp32c<KIND>(a, epi, sd, p, s0 - cc0, s1 - cc1, nn);
      }
      if (tid == 0) a.unit_done[ig] = 0;  // for the next pass
    }
  }
}

// ---------------------------------------------------------------------------
// FP32X passes.  The same CTA-per-cell staging, work split and pass-1 masks
// as FP32C, but each accepted candidate adds its fixed-point (cos phi_j,
// sin phi_j) (pass 2: d_j times those) to two 64-bit integer sums: exact,
// so the split of the list among warps, the order of the blocks and the
// staging rounds (added in 128 bits) do not change the result.  The kernel
// writes each particle's sums; k_epilogue_fp32x applies the angle addition
// and the stepper update in FP64.
constexpr int kTileCapX = 768;  // candidates staged per round (24 mask words)
static_assert(kTileCapX % 128 == 0 && kTileCapX / 32 <= kMaskWords, "FP32X staging round");

struct TileRedX {
  long long c[4][kTileThreads32], s[4][kTileThreads32];
  int n[4][kTileThreads32];
};

// One block of 32 staged candidates against one particle (FP32X): the float
// test, the fixed-point sums of the inside candidates, their bits, and the
// smallest |d^2 - mid| for the undecided check (as block32).
template <bool SELF>
__device__ __forceinline__ void block32x(const float2 *__restrict__ s_xy, const longlong2 *__restrict__ s_v,
                                         int j0, int self, float fxi, float fyi, float nmid, float nband,
                                         long long &C, long long &S, uint32_t &bits, float &mn) {
#pragma unroll
  for (int t = 0; t < kWarp; ++t) {
    const float2 cj = s_xy[j0 + t];
    const float dx = cj.x - fxi, dy = cj.y - fyi;
    float off = cutoff_offset(dx, dy, nmid);
    bool in = off < nband;
    if (SELF) {
      in = in && (j0 + t != self);
      off = (j0 + t != self) ? off : 3.0e38f;
    }
    mn = fminf(mn, fabsf(off));
    add2_if(C, S, s_v[j0 + t], in);
    bits |= (uint32_t)in << t;
  }
}

// Stage candidates [rlo, rlo + rcnt) of the stencil list (padded to rpad) for
// the FP32X passes (with part_fp32x, for the units kernel; the cell-tile
// kernel keeps the same code inline, as stage_fp32c says).
template <int KIND>
__device__ __forceinline__ void stage_fp32x(const KArgs &a, const SysConst &sc, const Stencil &st, int rlo,
                                            int rcnt, int rpad, float2 *s_xy, longlong2 *s_v) {
  for (int k = threadIdx.x; k < rpad; k += blockDim.x) {
    if (k < rcnt) {
      int q;
      const int pj = slot_of(st, rlo + k, q);
      const float2 f = a.fxy[pj];
      s_xy[k] = make_float2(f.x + shift_x(q, sc.cell_f), f.y + shift_y(q, sc.cell_f));
      s_v[k] = KIND == kKindSin ? a.ics[pj] : a.iws[pj];
    } else {  // padding: far away, never a neighbour, never near the cutoff
      s_xy[k] = make_float2(3.0e18f, 3.0e18f);
      s_v[k] = make_longlong2(0, 0);
    }
  }
}

// One warp: particle ig + li of a group of gi (lane li; li >= gi idle) against
// part [jlo, jhi) of the staged round [rlo, rlo + rcnt); its fixed-point sums
// and count go to red.*[part][li].  Called by all 32 lanes of the warp.
template <int KIND>
__device__ __forceinline__ void part_fp32x(const KArgs &a, const SysConst &sc, const Stencil &st,
                                           const float2 *s_xy, const longlong2 *s_v, TileRedX &red, int c0,
                                           int ig, int li, int gi, int rlo, int rcnt, int jlo, int jhi,
                                           int part, bool masked, bool exact_all, float band, float nmid) {
  const int n_all = a.n_active;
  const bool valid = li < gi;
  const int p = ig + li;
  float fxi = 3.0e30f, fyi = 3.0e30f;
  double xi = 0.0, yi = 0.0;
  if (valid) {
    const float2 f = a.fxy[p];
    fxi = f.x;
    fyi = f.y;
    xi = a.sx[p];
    yi = a.sy[p];
  }
  const int self = st.prefix[4] + (p - c0) - rlo;
  long long C = 0, Sn = 0;
  int n = 0;
  if (KIND == kKindCos2 && masked) {
    // pass 2 over the neighbour bitmask of pass 1 (same staged list)
    const uint4 *m4 = reinterpret_cast<const uint4 *>(a.nbmask);
    const uint4 none = make_uint4(0u, 0u, 0u, 0u);
    const int w0 = jlo / kWarp, w1 = jhi / kWarp;
    int g = w0 >> 2;
    uint4 cur = (valid && w0 < w1) ? m4[(size_t)g * n_all + p] : none;
    uint4 nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
    for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
      const int wd = j0 / kWarp;
      if ((wd >> 2) != g) {
        ++g;
        cur = nxt;
        nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
      }
      const int sub = wd & 3;
      const uint32_t bits = sub == 0 ? cur.x : sub == 1 ? cur.y : sub == 2 ? cur.z : cur.w;
#pragma unroll
      for (int t = 0; t < kWarp; ++t) {
        if ((bits >> t) & 1u) {
          const longlong2 v = s_v[j0 + t];
          C += v.x;
          Sn += v.y;
        }
      }
      n += __popc(bits);
    }
  } else {
    for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
      float mn = 3.0e38f;
      uint32_t bits = 0u;
      const bool self_block = (unsigned)(self - j0) < (unsigned)kWarp;
      if (!exact_all) {
        if (__any_sync(0xffffffffu, self_block))
          block32x<true>(s_xy, s_v, j0, self, fxi, fyi, nmid, -band, C, Sn, bits, mn);
        else
          block32x<false>(s_xy, s_v, j0, self, fxi, fyi, nmid, -band, C, Sn, bits, mn);
      }
      // pairs the float test cannot decide: the reference's FP64 test
      const bool amb = valid && (exact_all || mn <= band);
      if (__any_sync(0xffffffffu, amb)) {
        if (amb) {
          for (int t = 0; t < kWarp; ++t) {
            const int j = j0 + t;
            if (j == self || j >= rcnt) continue;
            const float2 cj = s_xy[j];
            const float dx = cj.x - fxi, dy = cj.y - fyi;
            if (!(exact_all || fabsf(cutoff_offset(dx, dy, nmid)) <= band)) continue;
            int q;
            const int pj = slot_of(st, rlo + j, q);
            if (!exact_within(sc, xi, yi, a.sx[pj], a.sy[pj])) continue;
            const longlong2 v = s_v[j];
            C += v.x;
            Sn += v.y;
            bits |= 1u << t;
          }
        }
      }
      n += __popc(bits);
      if (KIND == kKindSin && masked && valid) a.nbmask[mask_at(j0 / kWarp, p, n_all)] = bits;
    }
  }
  if (valid) {
    red.c[part][li] = C;
    red.s[part][li] = Sn;
    red.n[part][li] = n;
  }
}

// UNITS: unit cells are left to the units kernel (a separate instantiation, so
// that the kernel without cell units compiles exactly as before).
template <int KIND, bool UNITS>
__global__ void __launch_bounds__(kTileThreads32, kTileMinBlocks32) k_tile_fp32x(KArgs a, int epi) {
  __shared__ float2 s_xy[kTileCapX];     // x+shift, y+shift (padded to 32)
  __shared__ longlong2 s_v[kTileCapX];   // pass 1: ics, pass 2: iws of the candidate
  __shared__ TileRedX red;
  const int n_all = a.n_active;
  const int tid = threadIdx.x, w = tid / kWarp, lane = tid % kWarp;
  const int nitems = tile_items(a);
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    TileItem ti;
    if (!tile_item<kTileThreads32>(a, item, ti)) continue;
    if constexpr (UNITS) {
      if (a.cell_unit[ti.c]) continue;  // run by the units kernel
    }
    const int c = ti.c, c0 = ti.c0, cb = ti.cb, ce = ti.ce;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    Stencil st;
    stencil_of(a, sd, c, st);
    const int total = st.prefix[9];
    const int rounds = (total + kTileCapX - 1) / kTileCapX;
    const bool masked = rounds == 1 && a.nbmask != nullptr && !exact_all;
    for (int ig = cb; ig < ce; ig += kTileThreads32) {
      const int gi = min(kTileThreads32, ce - ig);
      // thread tid's particle (ig + tid): its sums over all rounds
      __int128 t_c = 0, t_s = 0;
      int t_n = 0;
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kTileCapX, rcnt = min(kTileCapX, total - rlo);
        const int rpad = (rcnt + kWarp - 1) & ~(kWarp - 1);
        if (rounds > 1 || ig == cb) {
          __syncthreads();
          for (int k = tid; k < rpad; k += blockDim.x) {
            if (k < rcnt) {
              int q;
              const int pj = slot_of(st, rlo + k, q);
              const float2 f = a.fxy[pj];
              s_xy[k] = make_float2(f.x + shift_x(q, sc.cell_f), f.y + shift_y(q, sc.cell_f));
              s_v[k] = KIND == kKindSin ? a.ics[pj] : a.iws[pj];
            } else {  // padding: far away, never a neighbour, never near the cutoff
              s_xy[k] = make_float2(3.0e18f, 3.0e18f);
              s_v[k] = make_longlong2(0, 0);
            }
          }
          __syncthreads();
        }
        const int chunks = (gi + kWarp - 1) / kWarp;
        const int S = chunks >= 4 ? 1 : (chunks == 1 ? 4 : 2);
        const int items = chunks * S;
        for (int item = w; item < items; item += kTileThreads32 / kWarp) {
          const int chunk = item / S, part = item % S;
          const int li = chunk * kWarp + lane;
          const bool valid = li < gi;
          const int p = ig + li;
          float fxi = 3.0e30f, fyi = 3.0e30f;
          double xi = 0.0, yi = 0.0;
          if (valid) {
            const float2 f = a.fxy[p];
            fxi = f.x;
            fyi = f.y;
            xi = a.sx[p];
            yi = a.sy[p];
          }
          const int self = st.prefix[4] + (p - c0) - rlo;
          const int jlo = split_point(rpad, part, S), jhi = split_point(rpad, part + 1, S);
          long long C = 0, Sn = 0;
          int n = 0;
          if (KIND == kKindCos2 && masked) {
            // pass 2 over the neighbour bitmask of pass 1 (same staged list)
            const uint4 *m4 = reinterpret_cast<const uint4 *>(a.nbmask);
            const uint4 none = make_uint4(0u, 0u, 0u, 0u);
            const int w0 = jlo / kWarp, w1 = jhi / kWarp;
            int g = w0 >> 2;
            uint4 cur = (valid && w0 < w1) ? m4[(size_t)g * n_all + p] : none;
            uint4 nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
            for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
              const int wd = j0 / kWarp;
              if ((wd >> 2) != g) {
                ++g;
                cur = nxt;
                nxt = (valid && ((g + 1) << 2) < w1) ? m4[(size_t)(g + 1) * n_all + p] : none;
              }
              const int sub = wd & 3;
              const uint32_t bits = sub == 0 ? cur.x : sub == 1 ? cur.y : sub == 2 ? cur.z : cur.w;
#pragma unroll
              for (int t = 0; t < kWarp; ++t) {
                if ((bits >> t) & 1u) {
                  const longlong2 v = s_v[j0 + t];
                  C += v.x;
                  Sn += v.y;
                }
              }
              n += __popc(bits);
            }
          } else {
            for (int j0 = jlo; j0 < jhi; j0 += kWarp) {
              float mn = 3.0e38f;
              uint32_t bits = 0u;
              const bool self_block = (unsigned)(self - j0) < (unsigned)kWarp;
              if (!exact_all) {
                if (__any_sync(0xffffffffu, self_block))
                  block32x<true>(s_xy, s_v, j0, self, fxi, fyi, nmid, -band, C, Sn, bits, mn);
                else
                  block32x<false>(s_xy, s_v, j0, self, fxi, fyi, nmid, -band, C, Sn, bits, mn);
              }
              // pairs the float test cannot decide: the reference's FP64 test
              const bool amb = valid && (exact_all || mn <= band);
              if (__any_sync(0xffffffffu, amb)) {
                if (amb) {
                  for (int t = 0; t < kWarp; ++t) {
                    const int j = j0 + t;
                    if (j == self || j >= rcnt) continue;
                    const float2 cj = s_xy[j];
                    const float dx = cj.x - fxi, dy = cj.y - fyi;
                    if (!(exact_all || fabsf(cutoff_offset(dx, dy, nmid)) <= band)) continue;
                    int q;
                    const int pj = slot_of(st, rlo + j, q);
                    if (!exact_within(sc, xi, yi, a.sx[pj], a.sy[pj])) continue;
                    const longlong2 v = s_v[j];
                    C += v.x;
                    Sn += v.y;
                    bits |= 1u << t;
                  }
                }
              }
              n += __popc(bits);
              if (KIND == kKindSin && masked && valid) a.nbmask[mask_at(j0 / kWarp, p, n_all)] = bits;
            }
          }
          if (valid) {
            red.c[part][li] = C;
            red.s[part][li] = Sn;
            red.n[part][li] = n;
          }
        }
        __syncthreads();
        if (tid < gi) {
          for (int part = 0; part < S; ++part) {
            t_c += red.c[part][tid];
            t_s += red.s[part][tid];
            t_n += red.n[part][tid];
          }
        }
      }
      if (tid < gi) {
        const int qv = KIND == kKindSin ? kXQ : sc.xq2;
        a.xsum[ig + tid] = make_double2(from_fixed128(t_c, qv), from_fixed128(t_s, qv));
        a.xcnt[ig + tid] = t_n;
      }
      __syncthreads();
    }
  }
}

// The units of an FP32X pass (listed by k_list_units after the gather),
// as k_units_fp32c.  A unit's round sums are exact 64-bit integers (below
// 2^62: kTileCapX candidates of |v| <= 2^52), added over the rounds in 128
// bits, so the particle's sums are those of the whole-group path.
template <int KIND>
__global__ void __launch_bounds__(kTileThreads32, kTileMinBlocks32) k_units_fp32x(KArgs a, int epi) {
  __shared__ float2 s_xy[kTileCapX];
  __shared__ longlong2 s_v[kTileCapX];
  __shared__ TileRedX red;
  __shared__ int s_last;
  const int n_all = a.n_active;
  const int tid = threadIdx.x, w = tid / kWarp, lane = tid % kWarp;
  const int count = *a.unit_count;
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const int2 e = a.units[i];
    // the unit's cell and, with sub-cells, its half: particles [g0, g1)
    const int c = a.cell_mid ? e.x >> 1 : e.x, half = a.cell_mid ? e.x & 1 : -1;
    const int c0 = a.cell_start[c];
    const int g0 = half == 1 ? a.cell_mid[c] : c0;
    const int g1 = half == 0 ? a.cell_mid[c] : a.cell_start[c + 1];
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    const int qv = KIND == kKindSin ? kXQ : sc.xq2;
    Stencil st;
    stencil_of(a, sd, c, st, half);
    const int total = st.prefix[9];
    const int rounds = (total + kTileCapX - 1) / kTileCapX;
    const bool masked = rounds == 1 && a.nbmask != nullptr && !exact_all;
    const int k = e.y / rounds, r = e.y - k * rounds;
    const int ig = g0 + k * kWarp, gi = min(kWarp, g1 - ig);
    const int rlo = r * kTileCapX, rcnt = min(kTileCapX, total - rlo);
    const int rpad = (rcnt + kWarp - 1) & ~(kWarp - 1);
    __syncthreads();
    stage_fp32x<KIND>(a, sc, st, rlo, rcnt, rpad, s_xy, s_v);
    __syncthreads();
    part_fp32x<KIND>(a, sc, st, s_xy, s_v, red, c0, ig, lane, gi, rlo, rcnt, split_point(rpad, w, 4),
                     split_point(rpad, w + 1, 4), w, masked, exact_all, band, nmid);
    __syncthreads();
    long long uc = 0, us = 0;
    int un = 0;
    if (tid < gi)
      for (int part = 0; part < 4; ++part) {
        uc += red.c[part][tid];
        us += red.s[part][tid];
        un += red.n[part][tid];
      }
    const int p = ig + tid;
    if (rounds == 1) {
      if (tid < gi) {
        a.xsum[p] = make_double2(from_fixed128(uc, qv), from_fixed128(us, qv));
        a.xcnt[p] = un;
      }
      continue;
    }
    if (tid < gi) {
      a.part_x[(size_t)r * n_all + p] = make_longlong2(uc, us);
      a.part_n[(size_t)r * n_all + p] = un;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&a.unit_done[ig], 1) == rounds - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      if (tid < gi) {
        __int128 sc_ = 0, ss_ = 0;
        int nn = 0;
        for (int q = 0; q < rounds; ++q) {
          const longlong2 v = __ldcg(&a.part_x[(size_t)q * n_all + p]);
          sc_ += v.x;
          ss_ += v.y;
          nn += __ldcg(&a.part_n[(size_t)q * n_all + p]);
        }
        a.xsum[p] = make_double2(from_fixed128(sc_, qv), from_fixed128(ss_, qv));
        a.xcnt[p] = nn;
      }
      if (tid == 0) a.unit_done[ig] = 0;  // for the next pass
    }
  }
}

// ---------------------------------------------------------------------------
template <int KIND>
__global__ void __launch_bounds__(kTileThreads64) k_tile_fp64(KArgs a, int epi) {
  __shared__ float2 s_xy[kTileCap64];   // x+shift, y+shift (prefilter)
  __shared__ double s_phi[kTileCap64];  // stage phase
  __shared__ double s_d[KIND == kKindCos2 ? kTileCap64 : 1];  // pass 2: phase rate
  __shared__ int s_p[kTileCap64];
  __shared__ uint16_t s_q[kQCap][kTileThreads64];
  const int tid = threadIdx.x;
  const int n_all = a.n_active;
  const int nitems = tile_items(a);
  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    TileItem ti;
    if (!tile_item<kTileThreads64>(a, item, ti)) continue;
    const int c = ti.c, c0 = ti.c0, cb = ti.cb, ce = ti.ce;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    Stencil st;
    stencil_of(a, sd, c, st);
    const int total = st.prefix[9];
    const int rounds = (total + kTileCap64 - 1) / kTileCap64;
    for (int ig = cb; ig < ce; ig += kTileThreads64) {
      const int gi = min(kTileThreads64, ce - ig);
      const bool valid = tid < gi;
      const int p = ig + tid;
      ILane il;
      load_i<kPrecFP64, KIND>(a, sc, il, p, valid);
      if (!valid) {
        il.fx = il.fy = 3.0e30f;
        il.x = il.y = il.phi = il.dphi = 0.0;
        il.card = il.rcard = 1.0;
      }
      Acc<kPrecFP64> acc;
      acc.init();
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kTileCap64, rcnt = min(kTileCap64, total - rlo);
        if (rounds > 1 || ig == cb) {
          __syncthreads();
          for (int k = tid; k < rcnt; k += blockDim.x) {
            int q;
            const int pj = slot_of(st, rlo + k, q);
            const float2 f = a.fxy[pj];
            s_xy[k] = make_float2(f.x + shift_x(q, sc.cell_f), f.y + shift_y(q, sc.cell_f));
            s_phi[k] = a.sphi[pj];
            s_p[k] = pj;
            if constexpr (KIND == kKindCos2) s_d[k] = a.dphi_s[pj];
          }
          __syncthreads();
        }
        const int self = st.prefix[4] + (p - c0) - rlo;
        int qn = 0, qh = 0;
        // accepted pair number `ord` of this particle (the same in both SRK
        // passes): single systems keep the first pass's cosine for the second
        // (sincos gives the bits of cos; spc_check_sincos)
        auto eval = [&](int j, int ord) {
          const double dphi_ = dsub(dsub(s_phi[j], il.phi), sc.alpha);
          double *slot = (a.tcos && ord < a.tcap) ? a.tcos + (size_t)ord * n_all + p : nullptr;
          if constexpr (KIND == kKindSin) {
            double sn;
            if (slot) {
              double cn;
              sincos(dphi_, &sn, &cn);
              *slot = cn;
            } else {
              sn = sin(dphi_);
            }
            acc.s0 = dadd(acc.s0, sn);  // ChimeraSystem.cpp:412
          } else {
            const double cc = slot ? *slot : cos(dphi_);  // ChimeraSystem.cpp:634-637
            acc.s0 = dadd(acc.s0, ddiv_by(cc, il.card, il.rcard));
            acc.s1 = dadd(acc.s1, ddiv_by(dmul(dsub(s_d[j], il.dphi), cc), il.card, il.rcard));
          }
        };
        for (int j0 = 0; j0 < rcnt; j0 += kWarp) {
          const int je = min(j0 + kWarp, rcnt);
          for (int j = j0; j < je; ++j) {
            const float2 cj = s_xy[j];
            const float off = cutoff_offset(cj.x - il.fx, cj.y - il.fy, nmid);
            bool in = !exact_all && float_inside(off, band) && (j != self);
            const bool amb = (exact_all || float_undecided(off, band)) && (j != self) && valid;
            if (__any_sync(0xffffffffu, amb)) {
              if (amb) in = exact_within(sc, il.x, il.y, a.sx[s_p[j]], a.sy[s_p[j]]);
            }
            if (in) {
              s_q[qn & (kQCap - 1)][tid] = (uint16_t)j;
              ++qn;
            }
          }
          // drain the warp's common backlog on full warps, in FIFO order (lanes
          // past the end of the cell hold no queue and do not bound it)
          int m = __reduce_min_sync(0xffffffffu, valid ? qn - qh : 0x7fffffff);
          if (m == 0x7fffffff) m = 0;
          if (valid) {
            for (int k = 0; k < m; ++k) eval(s_q[(qh + k) & (kQCap - 1)][tid], acc.n + qh + k);
            qh += m;
          }
          // keep room for the next block of 32
          while (qn - qh > kQCap - kWarp) {
            eval(s_q[qh & (kQCap - 1)][tid], acc.n + qh);
            ++qh;
          }
        }
        while (qh < qn) {  // tail of this round
          eval(s_q[qh & (kQCap - 1)][tid], acc.n + qh);
          ++qh;
        }
        acc.n += qn;
      }
      if (valid) epilogue<kPrecFP64, KIND>(a, epi, sd, il, acc, a.pidx[p]);
      __syncthreads();
    }
  }
}

}  // namespace spc
