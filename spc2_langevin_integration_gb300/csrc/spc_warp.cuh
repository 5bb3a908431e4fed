// Warp-per-cell neighbour passes for sparse cells.
//
// At the densities of ensembles of small systems a cell of side ~rho holds
// ~10 particles.  The cell-tile kernels (one CTA per cell, one thread per
// particle) then leave most lanes idle and, with one cell in flight per CTA,
// spend most of their time waiting on the cell's chain of dependent loads.
// Here one warp takes one cell, so ~4x more cells are in flight per SM.  The
// warp stages the cell's 3x3 stencil candidates in shared memory (the
// reference's visiting order, ChimeraSystem.cpp:39-44; ascending index inside
// a cell) with each stencil cell's periodic shift already added, and lane k
// loads particle k of the cell (32 at a time) for the epilogue.  Every pair is
// decided as in the other kernels: float prefilter on cell-relative
// coordinates, the reference's FP64 test in the band around rho^2.
//
// FP32C (k_warp_fp32c): the lanes are (particle, candidate group) pairs.  A
// chunk of g_n particles gets G = 32 / g_n groups; lane l works on particle
// l % g_n against the candidates j = group, group + G, ... of the staged list,
// so all lanes are busy even for cells of a few particles.  Each lane sums
// its accepted candidates' cos phi_j and sin phi_j per word of 32 candidates,
// turns them into the alignment terms by angle addition, and adds each word's
// term to a Kahan sum; the groups of one particle are combined in group order
// through shared memory.  Pass 1 stores each lane's accepted-candidate bits,
// pass 2 walks only those bits.
//
// FP64 (k_warp_fp64): for each particle i in turn the 32 lanes test 32
// candidates at a time; a ballot gives the neighbour word, the accepted
// candidates are compacted into a list, full warps of them evaluate sin / cos
// and the divisions in parallel, and lane i adds the values in list order, so
// every sum keeps the reference's order term for term (as the cell-tile FP64
// kernel does).
#pragma once

#include "spc_tile.cuh"

namespace spc {

constexpr int kWarpPassWarps = 4;
constexpr int kWarpPassThreads = kWarpPassWarps * kWarp;
constexpr int kWarpCap = 256;  // candidates staged per round (indices fit 8 bits)
// Cell-list systems with fewer particles per cell than this (on average) run
// the warp-per-cell passes by default.
constexpr double kSparseBelowDefault = 24.0;

// Candidates of the staging round [rlo, rlo + rcnt) into shared memory.
template <int PREC, int KIND>
__device__ __forceinline__ void stage_round(const KArgs &a, const SysConst &sc, const Stencil &st, int rlo,
                                            int rcnt, int lane, float4 *c4, float2 *xy, double *phi,
                                            float *df, double *dd) {
  for (int k = lane; k < rcnt; k += kWarp) {
    int q;
    const int pj = slot_of(st, rlo + k, q);
    const float2 f = a.fxy[pj];
    const float xs = f.x + shift_x(q, sc.cell_f), ys = f.y + shift_y(q, sc.cell_f);
    if constexpr (PREC == kPrecFP32C) {
      const float2 t = a.cs[pj];
      c4[k] = make_float4(xs, ys, t.x, t.y);
      if constexpr (KIND == kKindCos2) df[k] = a.dphi_f[pj];
    } else {
      xy[k] = make_float2(xs, ys);
      phi[k] = a.sphi[pj];
      if constexpr (KIND == kKindCos2) dd[k] = a.dphi_s[pj];
    }
  }
}

__device__ __forceinline__ void invalid_lane(ILane &il) {
  il.fx = il.fy = 3.0e30f;
  il.x = il.y = il.phi = il.dphi = 0.0;
  il.card = il.rcard = 1.0;
  il.ca = il.sa = il.dphif = 0.0f;
}

// ---------------------------------------------------------------------------
template <int KIND>
struct WarpStage32 {
  float4 c4[kWarpCap];  // x+shift, y+shift, cos phi, sin phi
  float df[KIND == kKindCos2 ? kWarpCap : 1];  // pass 2: phase rate (float)
  float s0[kWarp], c0[kWarp], s1[kWarp], c1[kWarp];  // per-lane partial sums
  int n[kWarp];
};

template <int KIND>
__global__ void __launch_bounds__(kWarpPassThreads, 8) k_warp_fp32c(KArgs a, int epi) {
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ WarpStage32<KIND> stage_all[kWarpPassWarps];
  const int w = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  WarpStage32<KIND> &sm = stage_all[w];
  const int n_all = a.n_active;
  const int stride = gridDim.x * kWarpPassWarps;
  for (int c = a.ncell_tile + blockIdx.x * kWarpPassWarps + w; c < a.va_c0; c += stride) {
    const int cb = a.cell_start[c], ce = a.cell_start[c + 1];
    if (cb == ce) continue;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    Stencil st;
    stencil_of(a, sd, c, st);
    const int total = st.prefix[9];
    const int rounds = (total + kWarpCap - 1) / kWarpCap;
    // one staging round: the lanes' candidate bits fit the particle's mask words
    const bool masked = rounds == 1 && a.nbmask != nullptr && !exact_all;
    for (int ib = cb; ib < ce; ib += kWarp) {
      const int gn = min(kWarp, ce - ib);
      const bool valid = lane < gn;
      ILane il;  // lane k: particle k of the chunk (load and epilogue)
      load_i<kPrecFP32C, KIND>(a, sc, il, ib + lane, valid);
      if (!valid) invalid_lane(il);
      // lane l: particle pl against candidate group g
      const int G = kWarp / gn, pl = lane % gn, g = lane / gn;
      const bool active = g < G;
      const float fxi = __shfl_sync(FULL, il.fx, pl), fyi = __shfl_sync(FULL, il.fy, pl);
      const float cai = __shfl_sync(FULL, il.ca, pl), sai = __shfl_sync(FULL, il.sa, pl);
      const float dfi = __shfl_sync(FULL, il.dphif, pl);
      const int pp = ib + pl;  // cell-order slot of the lane's particle
      float my_s0 = 0.0f, my_c0 = 0.0f, my_s1 = 0.0f, my_c1 = 0.0f;
      int my_n = 0;
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kWarpCap, rcnt = min(kWarpCap, total - rlo);
        const int self = st.prefix[4] + (pp - cb) - rlo;  // staged index of the lane's particle
        __syncwarp();
        if (rounds > 1 || ib == cb)
          stage_round<kPrecFP32C, KIND>(a, sc, st, rlo, rcnt, lane, sm.c4, nullptr, nullptr, sm.df, nullptr);
        __syncwarp();
        // words per lane: candidate k of the group sets bit k % 32 of word g * W + k / 32
        const int W = ((rcnt + G - 1) / G + kWarp - 1) / kWarp;
        float ps0 = 0.0f, pc0 = 0.0f, ps1 = 0.0f, pc1 = 0.0f;
        int pn = 0;
        if (active) {
          if (KIND == kKindCos2 && masked) {
            if constexpr (KIND == kKindCos2) {
              for (int wd = 0; wd < W; ++wd) {
                uint32_t bits = a.nbmask[mask_at(g * W + wd, pp, n_all)];
                pn += __popc(bits);
                float bc = 0.0f, bs = 0.0f, bdc = 0.0f, bds = 0.0f;
                while (bits) {
                  const int t = __ffs(bits) - 1;
                  bits &= bits - 1u;
                  const int j = g + (wd * kWarp + t) * G;
                  const float4 cj = sm.c4[j];
                  const float dj = sm.df[j];
                  bc += cj.z;
                  bs += cj.w;
                  bdc = fmaf(dj, cj.z, bdc);
                  bds = fmaf(dj, cj.w, bds);
                }
                // sum cos(phi_j - phi_i - alpha) and sum (d_j - d_i) cos(...)
                const float b0 = fmaf(bc, cai, bs * sai);
                kahan_add(ps0, pc0, b0);
                kahan_add(ps1, pc1, fmaf(bdc, cai, fmaf(bds, sai, -dfi * b0)));
              }
            }
          } else {
            uint32_t bits = 0u;
            int k = 0;
            float bc = 0.0f, bs = 0.0f, bdc = 0.0f, bds = 0.0f;  // this word's sums
            for (int j = g; j < rcnt; j += G, ++k) {
              const float4 cj = sm.c4[j];
              const float dx = cj.x - fxi, dy = cj.y - fyi;
              const float off = cutoff_offset(dx, dy, nmid);
              bool in = !exact_all && off < -band;
              if (exact_all || fabsf(off) <= band) {  // rare: the reference's FP64 test
                int q;
                const int pj = slot_of(st, rlo + j, q);
                in = exact_within(sc, a.sx[pp], a.sy[pp], a.sx[pj], a.sy[pj]);
              }
              in = in && j != self;
              if (in) {
                bits |= 1u << (k & (kWarp - 1));
                bc += cj.z;
                bs += cj.w;
                if constexpr (KIND == kKindCos2) {
                  const float dj = sm.df[j];
                  bdc = fmaf(dj, cj.z, bdc);
                  bds = fmaf(dj, cj.w, bds);
                }
              }
              if ((k & (kWarp - 1)) == kWarp - 1 || j + G >= rcnt) {
                // the word's alignment terms by angle addition (sin / cos of
                // phi_j - phi_i - alpha from cos phi_j, sin phi_j)
                if constexpr (KIND == kKindSin) {
                  kahan_add(ps0, pc0, fmaf(bs, cai, -bc * sai));
                } else {
                  const float b0 = fmaf(bc, cai, bs * sai);
                  kahan_add(ps0, pc0, b0);
                  kahan_add(ps1, pc1, fmaf(bdc, cai, fmaf(bds, sai, -dfi * b0)));
                }
                bc = bs = bdc = bds = 0.0f;
                pn += __popc(bits);
                if (KIND == kKindSin && masked) a.nbmask[mask_at(g * W + k / kWarp, pp, n_all)] = bits;
                bits = 0u;
              }
            }
            // a group with fewer candidates than group 0 leaves its last words empty
            if (KIND == kKindSin && masked)
              for (int wd = (k + kWarp - 1) / kWarp; wd < W; ++wd) a.nbmask[mask_at(g * W + wd, pp, n_all)] = 0u;
          }
        }
        // combine the groups of each particle in group order on its owner lane
        sm.s0[lane] = ps0;
        sm.c0[lane] = pc0;
        sm.s1[lane] = ps1;
        sm.c1[lane] = pc1;
        sm.n[lane] = pn;
        __syncwarp();
        if (valid) {
          for (int gg = 0; gg < G; ++gg) {
            const int src = gg * gn + lane;
            kahan_add(my_s0, my_c0, sm.s0[src]);
            kahan_add(my_s0, my_c0, -sm.c0[src]);
            if constexpr (KIND == kKindCos2) {
              kahan_add(my_s1, my_c1, sm.s1[src]);
              kahan_add(my_s1, my_c1, -sm.c1[src]);
            }
            my_n += sm.n[src];
          }
        }
      }
      if (valid) {
        Acc<kPrecFP32C> acc;
        acc.init();
        acc.s0 = my_s0 - my_c0;
        acc.s1 = my_s1 - my_c1;
        acc.n = my_n;
        epilogue<kPrecFP32C, KIND>(a, epi, sd, il, acc, a.pidx[ib + lane]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// FP32X: the lanes as in k_warp_fp32c; each lane adds its accepted
// candidates' fixed-point values (pass 1: cos phi_j, sin phi_j; pass 2: d_j
// times those) to two 64-bit integer sums, and the groups of a particle and
// the staging rounds are combined by integer adds (128 bits across rounds),
// so the sums are exact and independent of the grouping: bitwise those of
// the cell-tile kernel.  The kernel writes each particle's sums for
// k_epilogue_fp32x.
struct WarpStageX {
  float2 xy[kWarpCap];     // x+shift, y+shift
  longlong2 v[kWarpCap];   // pass 1: ics, pass 2: iws
  long long c[kWarp], s[kWarp];
  int n[kWarp];
};

template <int KIND>
__global__ void __launch_bounds__(kWarpPassThreads, 8) k_warp_fp32x(KArgs a, int epi) {
  __shared__ WarpStageX stage_all[kWarpPassWarps];
  const int w = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  WarpStageX &sm = stage_all[w];
  const int n_all = a.n_active;
  const int stride = gridDim.x * kWarpPassWarps;
  for (int c = a.ncell_tile + blockIdx.x * kWarpPassWarps + w; c < a.va_c0; c += stride) {
    const int cb = a.cell_start[c], ce = a.cell_start[c + 1];
    if (cb == ce) continue;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    const int qv = KIND == kKindSin ? kXQ : sc.xq2;
    Stencil st;
    stencil_of(a, sd, c, st);
    const int total = st.prefix[9];
    const int rounds = (total + kWarpCap - 1) / kWarpCap;
    const bool masked = rounds == 1 && a.nbmask != nullptr && !exact_all;
    for (int ib = cb; ib < ce; ib += kWarp) {
      const int gn = min(kWarp, ce - ib);
      const bool valid = lane < gn;
      // lane l: particle pl against candidate group g
      const int G = kWarp / gn, pl = lane % gn, g = lane / gn;
      const bool active = g < G;
      const int pp = ib + pl;
      const float2 fi = a.fxy[pp];
      const float fxi = fi.x, fyi = fi.y;
      __int128 my_c = 0, my_s = 0;  // lane k: particle k of the chunk, over all rounds
      int my_n = 0;
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kWarpCap, rcnt = min(kWarpCap, total - rlo);
        const int self = st.prefix[4] + (pp - cb) - rlo;
        __syncwarp();
        if (rounds > 1 || ib == cb) {
          for (int k = lane; k < rcnt; k += kWarp) {
            int q;
            const int pj = slot_of(st, rlo + k, q);
            const float2 f = a.fxy[pj];
            sm.xy[k] = make_float2(f.x + shift_x(q, sc.cell_f), f.y + shift_y(q, sc.cell_f));
            sm.v[k] = KIND == kKindSin ? a.ics[pj] : a.iws[pj];
          }
        }
        __syncwarp();
        const int W = ((rcnt + G - 1) / G + kWarp - 1) / kWarp;
        long long pc = 0, ps = 0;
        int pn = 0;
        if (active) {
          if (KIND == kKindCos2 && masked) {
            for (int wd = 0; wd < W; ++wd) {
              uint32_t bits = a.nbmask[mask_at(g * W + wd, pp, n_all)];
              pn += __popc(bits);
              while (bits) {
                const int t = __ffs(bits) - 1;
                bits &= bits - 1u;
                const longlong2 v = sm.v[g + (wd * kWarp + t) * G];
                pc += v.x;
                ps += v.y;
              }
            }
          } else {
            uint32_t bits = 0u;
            int k = 0;
            for (int j = g; j < rcnt; j += G, ++k) {
              const float2 cj = sm.xy[j];
              const float dx = cj.x - fxi, dy = cj.y - fyi;
              const float off = cutoff_offset(dx, dy, nmid);
              bool in = !exact_all && off < -band;
              if (exact_all || fabsf(off) <= band) {  // rare: the reference's FP64 test
                int q;
                const int pj = slot_of(st, rlo + j, q);
                in = exact_within(sc, a.sx[pp], a.sy[pp], a.sx[pj], a.sy[pj]);
              }
              in = in && j != self;
              bits |= (uint32_t)in << (k & (kWarp - 1));
              add2_if(pc, ps, sm.v[j], in);
              if ((k & (kWarp - 1)) == kWarp - 1 || j + G >= rcnt) {
                pn += __popc(bits);
                if (KIND == kKindSin && masked) a.nbmask[mask_at(g * W + k / kWarp, pp, n_all)] = bits;
                bits = 0u;
              }
            }
            // a group with fewer candidates than group 0 leaves its last words empty
            if (KIND == kKindSin && masked)
              for (int wd = (k + kWarp - 1) / kWarp; wd < W; ++wd) a.nbmask[mask_at(g * W + wd, pp, n_all)] = 0u;
          }
        }
        // combine the groups of each particle on its owner lane (integer adds)
        sm.c[lane] = pc;
        sm.s[lane] = ps;
        sm.n[lane] = pn;
        __syncwarp();
        if (valid) {
          for (int gg = 0; gg < G; ++gg) {
            const int src = gg * gn + lane;
            my_c += sm.c[src];
            my_s += sm.s[src];
            my_n += sm.n[src];
          }
        }
      }
      if (valid) {
        a.xsum[ib + lane] = make_double2(from_fixed128(my_c, qv), from_fixed128(my_s, qv));
        a.xcnt[ib + lane] = my_n;
      }
    }
  }
}

// ---------------------------------------------------------------------------
template <int KIND>
struct WarpStage64 {
  float2 xy[kWarpCap];  // x+shift, y+shift (prefilter)
  double phi[kWarpCap];
  double dd[KIND == kKindCos2 ? kWarpCap : 1];  // pass 2: phase rate
  uint8_t acc[2 * kWarp];                       // accepted candidates, in order
};

template <int KIND>
__global__ void __launch_bounds__(kWarpPassThreads) k_warp_fp64(KArgs a, int epi) {
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ WarpStage64<KIND> stage_all[kWarpPassWarps];
  const int w = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  WarpStage64<KIND> &sm = stage_all[w];
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int stride = gridDim.x * kWarpPassWarps;
  for (int c = a.ncell_tile + blockIdx.x * kWarpPassWarps + w; c < a.va_c0; c += stride) {
    const int cb = a.cell_start[c], ce = a.cell_start[c + 1];
    if (cb == ce) continue;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    Stencil st;
    stencil_of(a, sd, c, st);
    const int total = st.prefix[9];
    const int rounds = (total + kWarpCap - 1) / kWarpCap;
    for (int ib = cb; ib < ce; ib += kWarp) {
      const int gn = min(kWarp, ce - ib);
      const bool valid = lane < gn;
      const int p = ib + lane;
      ILane il;
      load_i<kPrecFP64, KIND>(a, sc, il, p, valid);
      if (!valid) invalid_lane(il);
      // this lane's particle: sums and neighbour count over all rounds
      double my_d0 = 0.0, my_d1 = 0.0;
      int my_n = 0;
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kWarpCap, rcnt = min(kWarpCap, total - rlo);
        const int nwords = (rcnt + kWarp - 1) / kWarp;
        __syncwarp();
        if (rounds > 1 || ib == cb)
          stage_round<kPrecFP64, KIND>(a, sc, st, rlo, rcnt, lane, nullptr, sm.xy, sm.phi, nullptr, sm.dd);
        __syncwarp();
        for (int i = 0; i < gn; ++i) {
          const float fxi = __shfl_sync(FULL, il.fx, i), fyi = __shfl_sync(FULL, il.fy, i);
          const int self = st.prefix[4] + (ib - cb) + i - rlo;  // staged index of i (may be outside)
          const double phii = __shfl_sync(FULL, il.phi, i);
          const double cardi = KIND == kKindCos2 ? __shfl_sync(FULL, il.card, i) : 1.0;
          const double rcardi = KIND == kKindCos2 ? __shfl_sync(FULL, il.rcard, i) : 1.0;
          const double dphii = KIND == kKindCos2 ? __shfl_sync(FULL, il.dphi, i) : 0.0;
          int n_i = 0, nacc = 0;
          // evaluate the first cnt listed candidates (one per lane) and add
          // them on lane i in list order
          auto flush = [&](int cnt) {
            double v0 = 0.0, v1 = 0.0;
            if (lane < cnt) {
              const int jj = sm.acc[lane];
              const double dp = dsub(dsub(sm.phi[jj], phii), sc.alpha);
              if constexpr (KIND == kKindSin) {
                v0 = sin(dp);  // ChimeraSystem.cpp:412
              } else {
                const double cc = cos(dp);  // ChimeraSystem.cpp:634-637
                v0 = ddiv_by(cc, cardi, rcardi);
                v1 = ddiv_by(dmul(dsub(sm.dd[jj], dphii), cc), cardi, rcardi);
              }
            }
            for (int k = 0; k < cnt; ++k) {
              const double t0 = __shfl_sync(FULL, v0, k);
              if (lane == i) my_d0 = dadd(my_d0, t0);
              if constexpr (KIND == kKindCos2) {
                const double t1 = __shfl_sync(FULL, v1, k);
                if (lane == i) my_d1 = dadd(my_d1, t1);
              }
            }
          };
          for (int wd = 0; wd < nwords; ++wd) {
            const int j = wd * kWarp + lane;
            bool in = false, amb = false;
            if (j < rcnt && j != self) {
              const float2 cj = sm.xy[j];
              const float off = cutoff_offset(cj.x - fxi, cj.y - fyi, nmid);
              in = !exact_all && float_inside(off, band);
              amb = exact_all || float_undecided(off, band);
            }
            if (amb) {  // rare: the reference's FP64 test
              int q;
              const int pj = slot_of(st, rlo + j, q);
              in = exact_within(sc, a.sx[ib + i], a.sy[ib + i], a.sx[pj], a.sy[pj]);
            }
            const uint32_t word = __ballot_sync(FULL, in);
            n_i += __popc(word);
            if (in) sm.acc[nacc + __popc(word & lt_mask)] = (uint8_t)j;
            nacc += __popc(word);
            if (nacc >= kWarp) {
              __syncwarp();
              flush(kWarp);
              const int rest = nacc - kWarp;
              const uint8_t tmp = lane < rest ? sm.acc[kWarp + lane] : (uint8_t)0;
              __syncwarp();
              if (lane < rest) sm.acc[lane] = tmp;
              __syncwarp();
              nacc = rest;
            }
          }
          if (nacc > 0) {
            __syncwarp();
            flush(nacc);
          }
          if (lane == i) my_n += n_i;
          __syncwarp();
        }
      }
      if (valid) {
        Acc<kPrecFP64> acc;
        acc.init();
        acc.s0 = my_d0;
        acc.s1 = my_d1;
        acc.n = my_n;
        epilogue<kPrecFP64, KIND>(a, epi, sd, il, acc, a.pidx[p]);
      }
    }
  }
}

}  // namespace spc
