// Verlet neighbour rows (ChimeraSystem::EvaluateInteractionsWithVerletNeighborList,
// ChimeraSystem.cpp:648-903; rebuild rule ChimeraSystemPtr.cpp:902-927).
//
// A build bins the stage positions into the rho-cells exactly as the cell-list
// path does (stage, radix sort, gather), which fixes a cell order, the
// "Verlet order" v, until the next build.  For every particle the build then
// lists, in the order of a (2R+1) x (2R+1) cell stencil (R = ceil(r_max / cell
// side), rows of cells top to bottom, ascending index inside a cell), every
// candidate within r_max = rho + skin of it.  A row entry is the candidate's
// index in the cell's staged stencil list (16 bits); rows are stored in
// chunks of 8 entries, chunk-major (chunk c of slot v is the 16 bytes at
// vrows[(c * n + v) * 8]), so one load gives a thread 8 entries and a warp's
// loads of one chunk are contiguous.
//
// Between builds an evaluation only refreshes the Verlet-order copies of the
// stage state (k_vgather, which also measures every particle's displacement
// from its build position) and walks the rows.  A pair within rho now was
// within rho + 2 * max displacement at the build, so while twice the largest
// displacement stays below the skin the rows hold every neighbour; the
// gather raises the rebuild flag before that can fail, and the rebuild
// kernels of the same evaluation (gated on that flag) rebuild the rows before
// the passes read them.  The passes decide every pair with the same float
// prefilter and exact FP64 cutoff test as the cell-list path, so neighbour
// sets are the reference's exactly; the summation order is the row order.
//
// A row longer than the row limit, or a stencil list longer than 65,535, is
// marked -1: that particle scans the whole staged stencil instead, which is
// still exact while the displacement bound holds.
#pragma once

#include "spc_tile.cuh"

namespace spc {

constexpr int kVThreads = 128;
constexpr int kVMaxR = 3;                 // stencil radius limit (7 x 7 cells)
constexpr int kVMaxCells = (2 * kVMaxR + 1) * (2 * kVMaxR + 1);
constexpr int kVStage32 = 1664;           // FP32C / build: candidates staged per round
constexpr int kVStage64 = 1536;           // FP64: candidates staged per round

// The (2R+1)^2 stencil of cell c: start of each stencil cell in cell order and
// the prefix offsets of the staged list, in shared memory.  All threads call it.
__device__ __forceinline__ void vstencil_of(const KArgs &a, const SysDesc &sd, int c, int *s_start,
                                            int *s_prefix) {
  const SysConst &sc = sd.sc;
  const int R = sc.vR, D = 2 * R + 1, nc = sc.nc;
  const int cl = c - sd.c0, cx = cl % nc, cy = cl / nc;
  __syncthreads();
  for (int q = threadIdx.x; q < D * D; q += blockDim.x) {
    const int ox = q % D - R, oy = q / D - R;
    const int jx = (cx + ox + nc) % nc, jy = (cy + oy + nc) % nc;  // nc >= 2R + 1
    const int cj = sd.c0 + jy * nc + jx;
    s_start[q] = a.cell_start[cj];
    s_prefix[q + 1] = a.cell_start[cj + 1] - a.cell_start[cj];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s_prefix[0] = 0;
    for (int q = 0; q < D * D; ++q) s_prefix[q + 1] += s_prefix[q];
  }
  __syncthreads();
}

// stencil entry of staged index g (binary search over the prefix table)
__device__ __forceinline__ int vstencil_entry(const int *s_prefix, int ncells, int g) {
  int lo = 0, hi = ncells - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (s_prefix[mid] <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Stage candidates [rlo, rlo + rcnt) of the stencil: prefilter coordinates
// relative to the centre cell's origin (and cos / sin, phase rate, phase as
// the pass needs them).
template <int PREC, int KIND, bool BUILD>
__device__ __forceinline__ void vstage_round(const KArgs &a, const SysConst &sc, const int *s_start,
                                             const int *s_prefix, int rlo, int rcnt, float4 *c4,
                                             float2 *xy, float *df, double *phi, double *dd) {
  const int R = sc.vR, D = 2 * R + 1;
  for (int k = threadIdx.x; k < rcnt; k += blockDim.x) {
    const int g = rlo + k;
    const int q = vstencil_entry(s_prefix, D * D, g);
    const int pj = s_start[q] + (g - s_prefix[q]);
    const float2 f = a.fxy[pj];
    const float xs = f.x + (float)(q % D - R) * sc.cell_f, ys = f.y + (float)(q / D - R) * sc.cell_f;
    if constexpr (BUILD || PREC == kPrecFP64) {
      xy[k] = make_float2(xs, ys);
    } else {
      const float2 t = a.cs[pj];
      c4[k] = make_float4(xs, ys, t.x, t.y);
    }
    if constexpr (!BUILD && PREC == kPrecFP32C && KIND == kKindCos2) df[k] = a.dphi_f[pj];
    if constexpr (!BUILD && PREC == kPrecFP64) {
      phi[k] = a.sphi[pj];
      if constexpr (KIND == kKindCos2) dd[k] = a.dphi_s[pj];
    }
  }
}

// entry `slot` (0..7) of a chunk of 8 row entries
__device__ __forceinline__ int chunk_entry(const uint4 &ch, int slot) {
  const uint32_t w = slot < 4 ? (slot < 2 ? ch.x : ch.y) : (slot < 6 ? ch.z : ch.w);
  return (int)((slot & 1) ? (w >> 16) : (w & 0xFFFFu));
}

// cell-order slot of staged index g (the exact-test fallback)
__device__ __forceinline__ int vslot_of(const SysConst &sc, const int *s_start, const int *s_prefix, int g) {
  const int D = 2 * sc.vR + 1;
  const int q = vstencil_entry(s_prefix, D * D, g);
  return s_start[q] + (g - s_prefix[q]);
}

// ---------------------------------------------------------------------------
// Build: rows of every particle of the cell (gated on vflags[0]).
__global__ void __launch_bounds__(kVThreads) k_verlet_build(KArgs a) {
  if (*a.gate == 0) return;
  __shared__ float2 s_xy[kVStage32];
  __shared__ int s_start[kVMaxCells], s_prefix[kVMaxCells + 1];
  const int n_all = a.n_active, tid = threadIdx.x;
  if (blockIdx.x == 0 && tid == 0) {
    a.vflags[1] = 0;  // a forced build is done
    atomicAdd(a.vrebuilds, 1ull);
  }
  for (int c = blockIdx.x; c < a.ncell_total; c += gridDim.x) {
    const int cb = a.cell_start[c], ce = a.cell_start[c + 1];
    if (cb == ce) continue;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    vstencil_of(a, sd, c, s_start, s_prefix);
    const int D = 2 * sc.vR + 1;
    const int total = s_prefix[D * D];
    const bool over = total > 65535;
    const int centre = s_prefix[sc.vR * D + sc.vR];
    const float r2 = sc.vr2;
    const int rounds = (total + kVStage32 - 1) / kVStage32;
    for (int ig = cb; ig < ce; ig += kVThreads) {
      const int v = ig + tid;
      const bool valid = v < ce;
      float fx = 0.0f, fy = 0.0f;
      if (valid) {
        const float2 f = a.fxy[v];
        fx = f.x;
        fy = f.y;
      }
      const int self = centre + (v - cb);
      int k = 0;
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kVStage32, rcnt = min(kVStage32, total - rlo);
        __syncthreads();
        vstage_round<kPrecFP64, kKindSin, true>(a, sc, s_start, s_prefix, rlo, rcnt, nullptr, s_xy,
                                                nullptr, nullptr, nullptr);
        __syncthreads();
        if (valid && !over) {
          for (int j = 0; j < rcnt; ++j) {
            const float2 cj = s_xy[j];
            const float dx = cj.x - fx, dy = cj.y - fy;
            if (fmaf(dx, dx, dy * dy) <= r2 && rlo + j != self) {
              if (k < a.vcap) a.vrows[((size_t)(k >> 3) * n_all + v) * 8 + (k & 7)] = (uint16_t)(rlo + j);
              ++k;
            }
          }
        }
      }
      if (valid) {
        a.vrowlen[v] = (!over && k <= a.vcap) ? k : -1;
        a.vxb[v] = a.sx[v];
        a.vyb[v] = a.sy[v];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Per evaluation: stage state of every Verlet slot from the pool (as k_stage:
// rk = s + (k_coef*dt) k_prev, ChimeraSystem.cpp:274-276, and the copy wrap,
// :299-302), prefilter coordinates relative to the slot's build cell (nearest
// periodic image), FP32C cos / sin, and the displacement test that raises the
// rebuild flag.  A forced build skips the work (the build tables are stale).
template <int PREC>
__global__ void __launch_bounds__(256) k_vgather(KArgs a, int rk_form, int kq, double kcdt) {
  __shared__ int s_any;
  const bool forced = a.vflags[1] != 0;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (!forced && v < a.n_active) {
    const SysDesc &sd = a.sys[a.vsys[v]];
    const SysConst &sc = sd.sc;
    const int q = a.pidx[v];
    double x = a.x[q], y = a.y[q], ph = a.phi[q];
    if (rk_form) {
      const double kx = kq >= 0 ? a.kx[kq][q] : 0.0;
      const double ky = kq >= 0 ? a.ky[kq][q] : 0.0;
      const double kp = kq >= 0 ? a.kphi[kq][q] : 0.0;
      x = dadd(x, dmul(kcdt, kx));
      y = dadd(y, dmul(kcdt, ky));
      ph = dadd(ph, dmul(kcdt, kp));
    }
    wrap_if_outside(sc, x, y);
    a.sx[v] = x;
    a.sy[v] = y;
    a.sphi[v] = ph;
    const int cl = a.vcell[v] - sd.c0, cx = cl % sc.nc, cy = cl / sc.nc;
    const double hL = 0.5 * sc.L;
    double dx = x - (double)cx * sc.cell, dy = y - (double)cy * sc.cell;
    dx = dx > hL ? dx - sc.L : (dx < -hL ? dx + sc.L : dx);
    dy = dy > hL ? dy - sc.L : (dy < -hL ? dy + sc.L : dy);
    a.fxy[v] = make_float2((float)dx, (float)dy);
    if constexpr (PREC == kPrecFP32C) {
      float s, c;
      sincosf(reduced_phase_f(ph), &s, &c);
      a.cs[v] = make_float2(c, s);
    }
    double ex = x - a.vxb[v], ey = y - a.vyb[v];
    ex = ex > hL ? ex - sc.L : (ex < -hL ? ex + sc.L : ex);
    ey = ey > hL ? ey - sc.L : (ey < -hL ? ey + sc.L : ey);
    if (ex * ex + ey * ey > sc.vdisp2) s_any = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0 && (s_any || forced)) atomicOr(&a.vflags[0], 1);
}

// ---------------------------------------------------------------------------
// Passes over the rows: one CTA per build cell, the cell's stencil staged in
// shared memory, one thread per particle walking its row (or, for an
// overflowed row, the whole staged list).
template <int PREC, int KIND>
struct VStage;

template <int KIND>
struct VStage<kPrecFP32C, KIND> {
  static constexpr int kCap = kVStage32;
  float4 c4[kCap];
  float df[KIND == kKindCos2 ? kCap : 1];
};

template <int KIND>
struct VStage<kPrecFP64, KIND> {
  static constexpr int kCap = kVStage64;
  float2 xy[kCap];
  double phi[kCap];
  double dd[KIND == kKindCos2 ? kCap : 1];
};

template <int PREC, int KIND>
__global__ void __launch_bounds__(kVThreads) k_vtile(KArgs a, int epi) {
  using Stage = VStage<PREC, KIND>;
  constexpr int kCap = Stage::kCap;
  __shared__ Stage sm;
  __shared__ int s_start[kVMaxCells], s_prefix[kVMaxCells + 1];
  const int n_all = a.n_active, tid = threadIdx.x;
  // the next evaluation's gather raises the flag again if it must
  if (blockIdx.x == 0 && tid == 0) a.vflags[0] = 0;
  for (int c = blockIdx.x; c < a.ncell_total; c += gridDim.x) {
    const int cb = a.cell_start[c], ce = a.cell_start[c + 1];
    if (cb == ce) continue;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const float lo2 = sc.lo2, hi2 = sc.hi2;
    const float band = 0.5f * (hi2 - lo2), nmid = -0.5f * (hi2 + lo2);
    const bool exact_all = sc.exact_all != 0;
    vstencil_of(a, sd, c, s_start, s_prefix);
    const int D = 2 * sc.vR + 1;
    const int total = s_prefix[D * D];
    const int centre = s_prefix[sc.vR * D + sc.vR];
    const int rounds = (total + kCap - 1) / kCap;
    for (int ig = cb; ig < ce; ig += kVThreads) {
      const int v = ig + tid;
      const bool valid = v < ce;
      ILane il;
      load_i<PREC, KIND>(a, sc, il, v, valid);
      const int len = valid ? a.vrowlen[v] : 0;
      const bool rows = len >= 0;
      // FP32C pass 2 reads pass 1's bits of row entries (rows only)
      const bool masked = PREC == kPrecFP32C && rows && a.nbmask != nullptr && !exact_all;
      const int self = centre + (v - cb);
      Acc<PREC> acc;
      acc.init();
      float b0 = 0.0f, b1 = 0.0f;  // FP32C: the current block of 32 entries
      uint32_t bits = 0u, word = 0u;
      int k = 0;  // entries (rows) or candidates (overflow) seen so far
      // rows: the chunk holding entry k and the next one (prefetched)
      const uint4 *chunks = reinterpret_cast<const uint4 *>(a.vrows);
      uint4 cur = make_uint4(0u, 0u, 0u, 0u), nextc = cur;
      int cur_chunk = 0;
      if (valid && rows && len > 0) {
        cur = chunks[v];
        if (len > 8) nextc = chunks[(size_t)n_all + v];
      }
      // one entry at staged offset j (round-relative) with global staged index g
      auto entry = [&](int j, int g) {
        bool in;
        if (KIND == kKindCos2 && masked) {
          if ((k & (kWarp - 1)) == 0) word = a.nbmask[(size_t)(k / kWarp) * n_all + v];
          in = (word >> (k & (kWarp - 1))) & 1u;
        } else {
          float cx, cy;
          if constexpr (PREC == kPrecFP32C) {
            const float4 cj = sm.c4[j];
            cx = cj.x;
            cy = cj.y;
          } else {
            const float2 cj = sm.xy[j];
            cx = cj.x;
            cy = cj.y;
          }
          const float off = cutoff_offset(cx - il.fx, cy - il.fy, nmid);
          in = !exact_all && float_inside(off, band);
          if (exact_all || float_undecided(off, band)) {  // rare: the reference's FP64 test
            const int pj = vslot_of(sc, s_start, s_prefix, g);
            in = exact_within(sc, il.x, il.y, a.sx[pj], a.sy[pj]);
          }
          in = in && g != self;
        }
        if (in) {
          if constexpr (PREC == kPrecFP32C) {
            const float4 cj = sm.c4[j];
            if constexpr (KIND == kKindSin) {
              b0 += fmaf(cj.w, il.ca, -cj.z * il.sa);  // sin(phi_j - phi_i - alpha)
            } else {
              const float tv = fmaf(cj.z, il.ca, cj.w * il.sa);  // cos(phi_j - phi_i - alpha)
              b0 += tv;
              b1 = fmaf(sm.df[j] - il.dphif, tv, b1);
            }
          } else {
            const double dp = dsub(dsub(sm.phi[j], il.phi), sc.alpha);
            // row entries only: k is then the entry's position in the row
            double *vc = (a.vcos && rows) ? a.vcos + (size_t)k * n_all + v : nullptr;
            if constexpr (KIND == kKindSin) {
              double sn, cn;
              if (vc) {  // keep the cosine for the second pass
                sincos(dp, &sn, &cn);
                *vc = cn;
              } else {
                sn = sin(dp);
              }
              acc.s0 = dadd(acc.s0, sn);  // ChimeraSystem.cpp:412
            } else {
              const double cc = vc ? *vc : cos(dp);  // ChimeraSystem.cpp:634-637
              acc.s0 = dadd(acc.s0, ddiv_by(cc, il.card, il.rcard));
              acc.s1 = dadd(acc.s1, ddiv_by(dmul(dsub(sm.dd[j], il.dphi), cc), il.card, il.rcard));
            }
          }
          bits |= 1u << (k & (kWarp - 1));
        }
        if ((k & (kWarp - 1)) == kWarp - 1) {  // close a block of 32 entries
          acc.n += __popc(bits);
          if constexpr (PREC == kPrecFP32C) {
            kahan_add(acc.s0, acc.c0, b0);
            if constexpr (KIND == kKindCos2) kahan_add(acc.s1, acc.c1, b1);
            b0 = b1 = 0.0f;
            if (KIND == kKindSin && masked) a.nbmask[(size_t)(k / kWarp) * n_all + v] = bits;
          }
          bits = 0u;
        }
        ++k;
      };
      for (int r = 0; r < rounds; ++r) {
        const int rlo = r * kCap, rcnt = min(kCap, total - rlo);
        __syncthreads();
        if constexpr (PREC == kPrecFP32C)
          vstage_round<PREC, KIND, false>(a, sc, s_start, s_prefix, rlo, rcnt, sm.c4, nullptr, sm.df,
                                          nullptr, nullptr);
        else
          vstage_round<PREC, KIND, false>(a, sc, s_start, s_prefix, rlo, rcnt, nullptr, sm.xy, nullptr,
                                          sm.phi, sm.dd);
        __syncthreads();
        if (!valid) continue;
        if (rows && rounds == 1 && !exact_all) {
          // the common case: every row entry is in the one staged round.
          // Chunks of 8 entries, unrolled, the next chunk loaded ahead.
          for (int c8 = 0; c8 * 8 < len; ++c8) {
            const uint4 ch = cur;
            if ((c8 + 1) * 8 < len) cur = chunks[(size_t)(c8 + 1) * n_all + v];
            if (KIND == kKindCos2 && masked && (c8 & 3) == 0)
              word = a.nbmask[(size_t)(c8 >> 2) * n_all + v];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              const int kk = c8 * 8 + t;
              if (kk < len) {
                const int j = chunk_entry(ch, t);
                bool in;
                if (KIND == kKindCos2 && masked) {
                  in = (word >> (kk & (kWarp - 1))) & 1u;
                } else {
                  float cx, cy;
                  if constexpr (PREC == kPrecFP32C) {
                    const float4 cj = sm.c4[j];
                    cx = cj.x;
                    cy = cj.y;
                  } else {
                    const float2 cj = sm.xy[j];
                    cx = cj.x;
                    cy = cj.y;
                  }
                  const float off = cutoff_offset(cx - il.fx, cy - il.fy, nmid);
                  in = float_inside(off, band);
                  if (float_undecided(off, band)) {  // rare: the reference's FP64 test
                    const int pj = vslot_of(sc, s_start, s_prefix, j);
                    in = exact_within(sc, il.x, il.y, a.sx[pj], a.sy[pj]);
                  }
                }
                if (in) {
                  if constexpr (PREC == kPrecFP32C) {
                    const float4 cj = sm.c4[j];
                    if constexpr (KIND == kKindSin) {
                      b0 += fmaf(cj.w, il.ca, -cj.z * il.sa);  // sin(phi_j - phi_i - alpha)
                    } else {
                      const float tv = fmaf(cj.z, il.ca, cj.w * il.sa);  // cos(phi_j - phi_i - alpha)
                      b0 += tv;
                      b1 = fmaf(sm.df[j] - il.dphif, tv, b1);
                    }
                  } else {
                    const double dp = dsub(dsub(sm.phi[j], il.phi), sc.alpha);
                    double *vc = a.vcos ? a.vcos + (size_t)kk * n_all + v : nullptr;
                    if constexpr (KIND == kKindSin) {
                      double sn, cn;
                      if (vc) {  // keep the cosine for the second pass
                        sincos(dp, &sn, &cn);
                        *vc = cn;
                      } else {
                        sn = sin(dp);
                      }
                      acc.s0 = dadd(acc.s0, sn);  // ChimeraSystem.cpp:412
                    } else {
                      const double cc = vc ? *vc : cos(dp);  // ChimeraSystem.cpp:634-637
                      acc.s0 = dadd(acc.s0, ddiv_by(cc, il.card, il.rcard));
                      acc.s1 = dadd(acc.s1, ddiv_by(dmul(dsub(sm.dd[j], il.dphi), cc), il.card, il.rcard));
                    }
                  }
                  bits |= 1u << (kk & (kWarp - 1));
                }
              }
            }
            if ((c8 & 3) == 3 && (c8 + 1) * 8 <= len) {  // a complete block of 32 entries
              acc.n += __popc(bits);
              if constexpr (PREC == kPrecFP32C) {
                kahan_add(acc.s0, acc.c0, b0);
                if constexpr (KIND == kKindCos2) kahan_add(acc.s1, acc.c1, b1);
                b0 = b1 = 0.0f;
                if (KIND == kKindSin && masked) a.nbmask[(size_t)(c8 >> 2) * n_all + v] = bits;
              }
              bits = 0u;
            }
          }
          k = len;
        } else if (rows) {
          // row entries are ascending staged indices: take those of this round
          while (k < len) {
            if ((k >> 3) != cur_chunk) {
              cur = nextc;
              ++cur_chunk;
              if ((cur_chunk + 1) * 8 < len) nextc = chunks[(size_t)(cur_chunk + 1) * n_all + v];
            }
            const int g = chunk_entry(cur, k & 7);
            if (g >= rlo + rcnt) break;
            entry(g - rlo, g);
          }
        } else {
          for (int j = 0; j < rcnt; ++j) entry(j, rlo + j);
        }
      }
      if (valid) {
        // the last, partial block
        acc.n += __popc(bits);
        if constexpr (PREC == kPrecFP32C) {
          kahan_add(acc.s0, acc.c0, b0);
          if constexpr (KIND == kKindCos2) kahan_add(acc.s1, acc.c1, b1);
          if (KIND == kKindSin && masked && (k & (kWarp - 1)) != 0)
            a.nbmask[(size_t)(k / kWarp) * n_all + v] = bits;
          acc.s0 = acc.s0 - acc.c0;
          acc.s1 = acc.s1 - acc.c1;
          acc.c0 = acc.c1 = 0.0f;
        }
        epilogue<PREC, KIND>(a, epi, sd, il, acc, a.pidx[v]);
      }
    }
  }
}

}  // namespace spc
