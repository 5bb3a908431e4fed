// Kernels of one right-hand-side evaluation and the fused stepper updates,
// for a batch of independent systems in one launch per phase.
//
// One evaluation (the reference's EvaluateInteractionsWithLinkedList,
// ChimeraSystem.cpp:258-426 / :429-645) runs as:
//   k_stage   stage state s + k_coef*dt*k_prev, copy-wrap, cell key  (ChimeraSystem.cpp:270-309)
//   sort      stable radix sort of (global cell key, index)           (:335-338)
//   k_gather  particles into cell order + float prefilter coordinates
//   k_tile_*  (spc_tile.cuh) one CTA per cell: the 3x3 stencil in the
//             reference's order, the exact FP64 cutoff, the alignment sums,
//             then a fused epilogue (k_next, or the whole stepper update with
//             noise and the engine's periodic wrap).
// When rho > L/4 the reference switches to all pairs (ChimeraSystem.cpp:90-98)
// on unwrapped stage positions; such a system is one "cell" here and
// k_allpairs_pass handles it.
//
// Indexing.  State (x, y, phi, omega, RK4 rates) lives in a particle pool:
// system s owns pool slots [pool_p0, pool_p0 + n).  Each evaluation works on
// the dense list of the active systems' particles, d in [0, n_active) with
// system s at [dense_p0, dense_p0 + n); after the sort, slot p in
// [0, n_active) is cell order.  Cells are global: system s owns cells
// [c0, c0 + nc^2) (one cell for an all-pairs system).  Per-system constants
// come from the SysDesc table, so a single system and a batch of hundreds run
// the same kernels.
#pragma once

#include "spc_device.cuh"
#include "spc_sort.cuh"

namespace spc {

enum { kPrecFP64 = 0, kPrecFP32C = 1, kPrecFP32X = 2 };
// what a pass accumulates over the neighbours of i
enum { kKindSin = 0, kKindCos2 = 1, kKindNb = 2 };
// what the pass does with the sums (runtime, warp-uniform)
enum Epilogue {
  kEpiRkK = 0,         // write k_next into k slot `kq_out` (RK form)
  kEpiRk4Combine = 1,  // k4, then the RK4 combine and the wrap
  kEpiEuler = 2,       // StochasticEulerStepper update + wrap
  kEpiSrk1 = 3,        // SRK pass 1: phase rate and n_i in cell order
  kEpiEulerPtr = 4,    // StochasticEulerStepperPtr update + wrap
  kEpiSrk2 = 5,        // SRK pass 2 and the strong-1.5 update + wrap
  kEpiSrk2Out = 6,     // SRK pass 2, derivative / additional_derivative out
  kEpiCount = 7,       // neighbour counts
  kEpiList = 8,        // neighbour indices in visiting order
  kEpiLocalOrder = 9,  // per-particle local order parameter
};

constexpr int kKSlots = 6;  // RK4 k1..k4 (persistent) + two scratch slots for spc_rhs_rk

// One system of a batch.
struct SysDesc {
  SysConst sc;
  int pool_p0;            // first pool slot
  int dense_p0;           // first dense index in the current layout
  int c0;                 // first global cell in the current layout
  int is_vortex;          // natural frequencies in the phase drift
  uint32_t system_id;     // Philox counter word
  uint64_t seed;          // Philox key
  unsigned long long step;     // steps taken before the current call (Philox counter)
  long long remaining;    // steps the system may still take (serving budget)
  int budget;             // steps of the current call it takes; later steps leave it frozen
};

struct KArgs {
  const SysDesc *sys;
  int nsys;
  int n_active;                      // dense particles
  int ncell_total;
  int ncell_tile;                    // cells [0, ncell_tile): cell-tile kernels
  int tile_split;                    // cell-tile kernels: CTAs per cell (0 or 1: one)
  int va_c0, va_c1;                  // [ncell_tile, va_c0): warp kernel; [va_c0, va_c1): vortex arrays
  const int *sys_of_p;               // dense index -> system
  const int *sys_of_c;               // global cell -> system
  // state pool (structure of arrays)
  double *x, *y, *phi;
  const double *omega;
  double *kx[kKSlots], *ky[kKSlots], *kphi[kKSlots];
  // stage (dense order)
  double *st_x, *st_y, *st_phi;
  uint32_t *keys, *vals;             // unsorted (global cell key, dense index)
  const uint32_t *skeys, *svals;     // sorted
  int *cell_start;
  // Sub-cells (SPC_TUNE_SUBCELLS; null when off): the sort key is 2c + h, h = 1
  // for the upper half of cell c (row_offset at least half a cell), and the
  // upper half starts at cell_mid[c].  cell_near[c] = 1 when a particle of
  // cell c lies within kNearHalf cell sides of the half line (cleared by
  // k_stage, set by k_gather).
  int *cell_mid;
  uint8_t *cell_near;
  // cell order
  double *sx, *sy, *sphi;
  float2 *fxy;                       // prefilter coordinates relative to the cell origin
  float2 *cs;                        // FP32C: (cos phi, sin phi)
  longlong2 *ics;                    // FP32X: (cos phi, sin phi) in fixed point (2^kXQ)
  longlong2 *iws;                    // FP32X SRK: phase rate times (cos phi, sin phi), fixed point (2^xq2)
  double *scos;                      // FP32X SRK: pass-1 sum_j cos(phi_j - phi_i - alpha), cell order
  double2 *xsum;                     // FP32X: a pass's exact neighbour sums (c, s), cell order
  int *xcnt;                         // FP32X: a pass's neighbour count, cell order
  int *pidx;                         // pool slot of cell-order slot p
  double *dphi_s;                    // SRK pass 1 phase rate, cell order
  float *dphi_f;                     // same, float (FP32C)
  int *cnt_s;                        // n_i, cell order
  double *va_vx, *va_vy;             // vortex arrays: pass-1 velocity components, cell order
  int *va_cnt2;                      // vortex arrays: cohesion partners, cell order
  uint32_t *nbmask;                  // FP32C: pass-1 neighbour bitmasks (mask_at), or null
  // Cell units of the float cell-tile passes (SPC_TUNE_CELL_UNITS; units
  // null when off): the units k_list_units lists for the units kernel
  // (cell, unit), their count (zeroed by k_gather), per staging
  // round r and cell-order slot p at [r * n_active + p] a unit's sums (FP32C:
  // float pair, FP32X: fixed-point pair) and counts, and a completion counter
  // per 32-particle chunk, indexed by its first slot (zero between launches).
  int2 *units;
  int *unit_count;
  uint8_t *cell_unit;  // per cell-tile cell: 1 if it runs as units (written with the list)
  float2 *part_f;
  longlong2 *part_x;
  int *part_n;
  int *unit_done;
  uint32_t *hist;                    // radix histogram table (zeroed by k_gather)
  int hist_len;
  const int *ap_cells;               // global cells of the all-pairs systems
  int n_ap;
  // parity / diagnostics outputs, indexed by pool slot
  double *out_d, *out_a, *out_r;
  int *out_cnt;
  const long long *list_off;
  int *list_idx;
  // stepping
  double dt;
  double sdt;                        // sqrt(dt), rounded once on the host
  int kq_out;                        // k slot written by kEpiRkK / kEpiRk4Combine (k4)
  const double *noise;               // injected normals of this step (pool-indexed), or null
  int noise_m;                       // normals per particle
  int step_off;                      // this step = sys.step + step_off
  unsigned long long *clamped;
  // Verlet rows (null / 0 on the cell-list path)
  const int *gate;                   // binning kernels return at once when *gate == 0
  int *vsys, *vcell;                 // build: system and cell of each cell-order slot
  uint16_t *vrows;                   // row entry k of slot v at vrows[((k / 8) * n_active + v) * 8 + k % 8]
  double *vcos;                      // FP64 SRK: cos of row entry k's phase difference at vcos[k * n_active + v], or null
  // vortex-arrays SRK (single systems): the first pass's record of slot p's
  // k-th pair within rho (k < vacap): strength, its derivative, sin and cos of
  // the phase difference at vacache[(k * n_active + p) * 4 + 0..3], or null
  double *vacache;
  int vacap;
  // cell-tile FP64 SRK (single systems): cos of slot p's k-th accepted pair
  // (k < tcap) from the first pass at tcos[k * n_active + p], or null
  double *tcos;
  int tcap;
  int *vrowlen;                      // entries of each row, -1: overflow (scan the stencil)
  int vcap;                          // row limit of the current build
  double *vxb, *vyb;                 // stage positions at the build
  int *vflags;                       // [0] rebuild needed this evaluation, [1] forced
  unsigned long long *vrebuilds;
};

// Global cell of cell-order slot p (its sort key, halved with sub-cells).
__device__ __forceinline__ int cell_of_slot(const KArgs &a, int p) {
  const int k = (int)a.skeys[p];
  return a.cell_mid ? k >> 1 : k;
}

// Sub-cells: a stage y's offset above the lower edge of its cell row cy.  It
// decides the half (upper when >= cell / 2) in k_stage and the near flag in
// k_gather, the same expression in both.
__device__ __forceinline__ double row_offset(const SysConst &sc, double y, int cy) {
  return dsub(y, dmul((double)cy, sc.cell));
}

// A half's stencil leaves out the far half of the row beyond it.  The pairs
// left out are more than a cell side (>= rho) apart unless both particles
// lie within rounding of the half line, so each cell records whether any of
// its particles lies within kNearHalf cell sides of the line, and a far cell
// stays whole when both it and the half's own cell do.  2^-20 of a cell is
// far above the rounding of the row offsets and of the reference's distance
// (a few ulps of L, L < 2^30 cells), and holds ~2e-6 of the particles.
constexpr double kNearHalf = 0x1p-20;

// ---------------------------------------------------------------------------
// k_stage: rk = s + (k_coef*dt) * k_prev (ChimeraSystem.cpp:274-276), the copy
// wrap and cell key (:295-308).  kq < 0 means k_prev is all zeros (the Euler
// stepper's zero-filled buffer, StochasticEulerStepper.hpp:34); rk_form = 0 is
// the SRK form, whose stage state is the state itself (:456-458).  With
// sub-cells the key also carries the half of the cell (the upper half when
// the stage y is at least half a cell above the cell's lower edge).
// With hist_bits > 0 the kernel also counts the first radix digit per sort
// tile into hist (tile-major [tile][digit], zero on entry): a block-local
// shared histogram, then one global atomic per non-empty bin.
constexpr int kStageThreads = 256;

constexpr int kMaxHistBits = 11;

__global__ void __launch_bounds__(kStageThreads)
    k_stage(KArgs a, int rk_form, int kq, double kcdt, int hist_bits, uint32_t *hist) {
  if (a.gate && *a.gate == 0) return;
  __shared__ uint32_t h[1 << kMaxHistBits];
  const int R = 1 << hist_bits;
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (hist_bits > 0) {
    for (int k = threadIdx.x; k < R; k += blockDim.x) h[k] = 0;
    __syncthreads();
  }
  if (a.cell_mid)  // this evaluation's near flags (set by k_gather)
    for (int c = d; c < a.ncell_total; c += gridDim.x * blockDim.x) a.cell_near[c] = 0;
  if (d < a.n_active) {
    const SysDesc &sd = a.sys[a.sys_of_p[d]];
    const SysConst &sc = sd.sc;
    const int q = sd.pool_p0 + (d - sd.dense_p0);
    double x = a.x[q], y = a.y[q], ph = a.phi[q];
    if (rk_form) {
      const double kx = kq >= 0 ? a.kx[kq][q] : 0.0;
      const double ky = kq >= 0 ? a.ky[kq][q] : 0.0;
      const double kp = kq >= 0 ? a.kphi[kq][q] : 0.0;
      x = dadd(x, dmul(kcdt, kx));
      y = dadd(y, dmul(kcdt, ky));
      ph = dadd(ph, dmul(kcdt, kp));
    }
    uint32_t key;
    if (sc.allpairs) {
      // all pairs use the unwrapped stage positions (ChimeraSystem.cpp:135-153)
      key = a.cell_mid ? 2u * (uint32_t)sd.c0 : (uint32_t)sd.c0;
    } else {
      wrap_if_outside(sc, x, y);
      int clamped = 0;
      const int cx = cell_coord(sc, x, clamped);
      const int cy = cell_coord(sc, y, clamped);
      if (clamped) atomicAdd(a.clamped, 1ull);
      key = (uint32_t)(sd.c0 + cy * sc.nc + cx);
      if (a.cell_mid) key = 2u * key + (row_offset(sc, y, cy) >= 0.5 * sc.cell ? 1u : 0u);
    }
    a.st_x[d] = x;
    a.st_y[d] = y;
    a.st_phi[d] = ph;
    a.keys[d] = key;
    a.vals[d] = (uint32_t)d;
    if (hist_bits > 0) atomicAdd(&h[key & (R - 1)], 1u);
  }
  if (hist_bits > 0) {
    __syncthreads();
    // a block of 256 lies inside one sort tile of 2048
    uint32_t *row = hist + (size_t)(blockIdx.x * blockDim.x / kSortTile) * R;
    for (int k = threadIdx.x; k < R; k += blockDim.x)
      if (h[k]) atomicAdd(&row[k], h[k]);
  }
}

// Phase reduced to about [-pi, pi] in double, then float (FP32C trig input).
__device__ __forceinline__ float reduced_phase_f(double ph) {
  const double two_pi = 6.283185307179586;
  const double inv_two_pi = 0.15915494309189535;
  return (float)(ph - two_pi * rint(ph * inv_two_pi));
}

template <int PREC>
__global__ void k_gather(KArgs a) {
  if (a.gate && *a.gate == 0) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.n_active;
  if (p > n) return;
  // the cell start table of the sorted keys (one thread per slot and one past the end)
  if (a.cell_mid)
    half_bounds_at(a.skeys, n, a.ncell_total, a.cell_start, a.cell_mid, p);
  else
    cell_bounds_at(a.skeys, n, a.ncell_total, a.cell_start, p);
  // leave the first-digit histogram table zero for the next stage kernel
  for (int k = p; k < a.hist_len; k += n + 1) a.hist[k] = 0u;
  if (p == n) {
    if (a.unit_count) *a.unit_count = 0;  // this evaluation's cell units (k_list_units)
    return;
  }
  const int d = (int)a.svals[p];
  const SysDesc &sd = a.sys[a.sys_of_p[d]];
  const SysConst &sc = sd.sc;
  const double x = a.st_x[d], y = a.st_y[d], ph = a.st_phi[d];
  a.sx[p] = x;
  a.sy[p] = y;
  a.sphi[p] = ph;
  a.pidx[p] = sd.pool_p0 + (d - sd.dense_p0);
  if (a.vsys) {  // Verlet build: remember each slot's system and cell until the next build
    a.vsys[p] = a.sys_of_p[d];
    a.vcell[p] = cell_of_slot(a, p);
  }
  if (!sc.allpairs) {
    const int key = cell_of_slot(a, p) - sd.c0;
    const int cx = key % sc.nc, cy = key / sc.nc;
    a.fxy[p] = make_float2((float)(x - (double)cx * sc.cell), (float)(y - (double)cy * sc.cell));
    if (a.cell_mid && fabs(row_offset(sc, y, cy) - 0.5 * sc.cell) < kNearHalf * sc.cell)
      a.cell_near[sd.c0 + key] = 1;
  }
  if constexpr (PREC == kPrecFP32C) {
    float s, c;
    sincosf(reduced_phase_f(ph), &s, &c);
    a.cs[p] = make_float2(c, s);
  }
  if constexpr (PREC == kPrecFP32X) {
    double s, c;
    sincos(ph, &s, &c);
    a.ics[p] = make_longlong2(to_fixed(c, kXQ), to_fixed(s, kXQ));
  }
}

// ---------------------------------------------------------------------------
// Per-i accumulators of one pass.
template <int PREC>
struct Acc;

template <>
struct Acc<kPrecFP64> {
  double s0, s1;  // sin sum | cos/n sum, (dphi) cos/n sum | cos, sin sums
  int n;
  __device__ void init() { s0 = 0.0; s1 = 0.0; n = 0; }
};

template <>
struct Acc<kPrecFP32C> {
  float s0, c0, s1, c1;  // Kahan sums and compensations
  int n;
  __device__ void init() { s0 = c0 = s1 = c1 = 0.0f; n = 0; }
};

// Word w (< 32) of the pass-1 neighbour bitmask of cell-order slot p among n
// active particles.  Four consecutive words of a particle share one 16-byte
// group.  The cell-tile and warp-per-cell kernels of one pass write the same
// buffer for the particles of their own cells, so both must index it this way:
// distinct (w, p) never share a word.  (The Verlet kernels keep a word-major
// layout of their own; a Verlet engine holds one system and runs no other
// neighbour kernel in the pass.)
__device__ __forceinline__ size_t mask_at(int w, int p, int n) {
  return ((size_t)(w >> 2) * n + p) * 4 + (w & 3);
}

// Float prefilter offset d^2 - mid of a candidate at (dx, dy), in two fused
// multiply-adds.  A pair is inside when off < -band, outside when off > band,
// and undecided (left to the reference's FP64 test) otherwise: one value for
// all three, so the float-inside and undecided sets are disjoint.  Float
// error is ~1e-7 rho^2, far inside the band of 3e-5 rho^2.
__device__ __forceinline__ float cutoff_offset(float dx, float dy, float nmid) {
  return fmaf(dx, dx, fmaf(dy, dy, nmid));
}

// Every neighbour kernel decides a candidate from that one offset: inside when
// off < -band, undecided (the reference's FP64 test decides) when
// |off| <= band, outside otherwise.  The inside and undecided sets are then
// disjoint and leave no gap below mid + band.  Deciding instead from d^2 < lo2
// and |d^2 - mid| <= band separately leaves one: mid = (lo2 + hi2) / 2 is
// rounded, and for about one rho in five |lo2 - mid| exceeds band by a
// fraction of an ulp, so a float d^2 equal to lo2 is in neither set and a pair
// just inside the cutoff (d^2 ~ rho^2 (1 - 3e-5)) is dropped.
__device__ __forceinline__ bool float_inside(float off, float band) { return off < -band; }
__device__ __forceinline__ bool float_undecided(float off, float band) { return fabsf(off) <= band; }

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float v) {
  const float y = v - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// Everything an i lane needs inside the candidate loop.
struct ILane {
  int p;        // cell-order slot
  bool valid;
  float fx, fy; // prefilter coordinates
  double x, y;  // wrapped stage position
  double phi;   // stage phase
  double card;  // pass 2: n_i from pass 1 (double, as neighborhood_cardinality_)
  double rcard; // pass 2: 1 / n_i rounded to nearest (ddiv_by)
  double dphi;  // pass 2: own phase rate
  float ca, sa; // FP32C: cos(phi + alpha), sin(phi + alpha)
  float dphif;
};

template <int PREC, int KIND>
__device__ __forceinline__ void accept_pair(const KArgs &a, const SysDesc &sd, const ILane &il,
                                            Acc<PREC> &acc, int pj, float cjc, float cjs,
                                            float dphij_f, long long &wpos) {
  const SysConst &sc = sd.sc;
  if constexpr (KIND == kKindSin) {
    if constexpr (PREC == kPrecFP64) {
      // alignment_force_[i] += sin(phi_j - phi_i - alpha_) (ChimeraSystem.cpp:412)
      acc.s0 = dadd(acc.s0, sin(dsub(dsub(a.sphi[pj], il.phi), sc.alpha)));
    } else {
      // sin(phi_j - (phi_i + alpha)) by the angle-difference identity
      kahan_add(acc.s0, acc.c0, cjs * il.ca - cjc * il.sa);
    }
    acc.n++;
  } else if constexpr (KIND == kKindCos2) {
    if constexpr (PREC == kPrecFP64) {
      // ChimeraSystem.cpp:634-637
      const double c = cos(dsub(dsub(a.sphi[pj], il.phi), sc.alpha));
      acc.s0 = dadd(acc.s0, ddiv_by(c, il.card, il.rcard));
      acc.s1 = dadd(acc.s1, ddiv_by(dmul(dsub(a.dphi_s[pj], il.dphi), c), il.card, il.rcard));
    } else {
      const float c = cjc * il.ca + cjs * il.sa;
      kahan_add(acc.s0, acc.c0, c);
      kahan_add(acc.s1, acc.c1, (dphij_f - il.dphif) * c);
    }
    acc.n++;
  } else {
    if (a.list_idx) a.list_idx[wpos++] = a.pidx[pj] - sd.pool_p0;
    if constexpr (PREC == kPrecFP64) {
      if (a.out_r) {
        acc.s0 += cos(a.sphi[pj]);
        acc.s1 += sin(a.sphi[pj]);
      }
    }
    acc.n++;
  }
}

__device__ __forceinline__ double noise_at(const KArgs &a, int q, int k, double z0, double z1) {
  if (a.noise) return a.noise[(size_t)q * a.noise_m + k];
  return k == 0 ? z0 : z1;
}

// Fused epilogue for the particle in pool slot q (system sd) at cell-order slot p.
template <int PREC, int KIND>
__device__ void epilogue(const KArgs &a, int epi, const SysDesc &sd, const ILane &il,
                         Acc<PREC> &acc, int q, const double2 *cs_known = nullptr) {
  const SysConst &sc = sd.sc;
  const int p = il.p;
  if constexpr (KIND == kKindNb) {
    if (epi == kEpiCount) a.out_cnt[q] = acc.n;
    if (epi == kEpiLocalOrder) {
      const double re = acc.s0 + cos(il.phi), im = acc.s1 + sin(il.phi);
      a.out_r[q] = sqrt(re * re + im * im) / (double)(acc.n + 1);
    }
    return;
  }
  // past its step budget a system is frozen: no persistent state changes
  const bool live = a.step_off < sd.budget;
  const int i = q - sd.pool_p0;  // index within the system (Philox counter)
  const unsigned long long step = sd.step + (unsigned long long)a.step_off;
  double z0 = 0.0, z1 = 0.0;
  const bool draws = (epi == kEpiEuler || epi == kEpiEulerPtr || epi == kEpiSrk2) && !a.noise && live;
  const double dt = a.dt;
  if constexpr (PREC == kPrecFP64) {
    if (draws) philox_normal2(sd.seed, sd.system_id, step, (uint32_t)i, z0, z1);
    // cos / sin of the stage phase: evaluated here, or (FP32X) the gather's
    // fixed-point values, exact to 2^-53
    const double cph = cs_known ? cs_known->x : cos(il.phi), sph = cs_known ? cs_known->y : sin(il.phi);
    const double d0 = dmul(sc.v0, cph), d1 = dmul(sc.v0, sph);  // v_0_ * cos(phi_i) (:419-420)
    if constexpr (KIND == kKindSin) {
      // sigma_ * alignment_force_[i] / neighborhood_cardinality_[i] (:421-424)
      const bool has = acc.n != 0;
      const double rate = has ? ddiv(dmul(sc.sigma, acc.s0), (double)acc.n) : 0.0;
      if (epi == kEpiRkK || epi == kEpiRk4Combine) {
        if (!live) return;
        const int k = a.kq_out;
        a.kx[k][q] = d0;
        a.ky[k][q] = d1;
        if (has) a.kphi[k][q] = rate;  // otherwise k_next keeps its value (H5)
        if (epi == kEpiRk4Combine) {
          // RungeKutta4Stepper.cpp:52-54
          const double k4p = a.kphi[k][q];
          double xs = a.x[q], ys = a.y[q], ps = a.phi[q];
          const double sx_ = dadd(dadd(dadd(a.kx[0][q], dmul(2.0, a.kx[1][q])), dmul(2.0, a.kx[2][q])), d0);
          const double sy_ = dadd(dadd(dadd(a.ky[0][q], dmul(2.0, a.ky[1][q])), dmul(2.0, a.ky[2][q])), d1);
          const double sp_ = dadd(dadd(dadd(a.kphi[0][q], dmul(2.0, a.kphi[1][q])), dmul(2.0, a.kphi[2][q])), k4p);
          xs = dadd(xs, ddiv(dmul(sx_, dt), 6.0));
          ys = dadd(ys, ddiv(dmul(sy_, dt), 6.0));
          ps = dadd(ps, dmul(ddiv(sp_, 6.0), dt));
          a.x[q] = wrap_1d(xs, sc.rL, sc.L);  // SimulationEngine.cpp:154
          a.y[q] = wrap_1d(ys, sc.rL, sc.L);
          a.phi[q] = ps;
        }
      } else if (epi == kEpiEuler) {
        if (!live) return;
        // StochasticEulerStepper.hpp:43-45 with AddNoise (ChimeraSystem.cpp:927-930);
        // a vortex system adds its frequency to the phase drift as the
        // SRK-Ptr stepper does (StochasticRungeKuttaStepperPtr.hpp:65)
        const double sdt = a.sdt;
        const double sto = dmul(sc.s2D, noise_at(a, q, 0, z0, z1));
        const double xs = dadd(a.x[q], dadd(dmul(dt, d0), dmul(sdt, 0.0)));
        const double ys = dadd(a.y[q], dadd(dmul(dt, d1), dmul(sdt, 0.0)));
        const double drift = sd.is_vortex ? dadd(a.omega[q], rate) : rate;
        a.phi[q] = dadd(a.phi[q], dadd(dmul(dt, drift), dmul(sdt, sto)));
        a.x[q] = wrap_1d(xs, sc.rL, sc.L);
        a.y[q] = wrap_1d(ys, sc.rL, sc.L);
      } else if (epi == kEpiEulerPtr) {
        if (!live) return;
        // StochasticEulerStepperPtr.hpp:44-51
        const double dW = dmul(a.sdt, noise_at(a, q, 0, z0, z1));
        const double xs = dadd(a.x[q], dmul(d0, dt));
        const double ys = dadd(a.y[q], dmul(d1, dt));
        a.phi[q] = dadd(a.phi[q], dadd(dmul(rate, dt), dmul(sc.s2D, dW)));
        a.x[q] = wrap_1d(xs, sc.rL, sc.L);
        a.y[q] = wrap_1d(ys, sc.rL, sc.L);
      } else if (epi == kEpiSrk1) {
        a.dphi_s[p] = rate;  // derivative is zero-filled each step: 0 when isolated
        a.cnt_s[p] = acc.n;
      }
    } else {  // kKindCos2: SRK pass 2 (ChimeraSystem.cpp:642-643)
      const double A0 = dmul(acc.s0, -sc.s2D);
      const double A1 = dadd(acc.s1, dmul(dmul(-2.0, sc.D), il.dphi));
      const double d2 = il.dphi;
      if (epi == kEpiSrk2Out) {
        a.out_d[3 * (size_t)q] = d0;
        a.out_d[3 * (size_t)q + 1] = d1;
        a.out_d[3 * (size_t)q + 2] = d2;
        a.out_a[2 * (size_t)q] = A0;
        a.out_a[2 * (size_t)q + 1] = A1;
      } else {
        if (!live) return;
        // StochasticRungeKuttaStepper.hpp:44-55 (+ omega: StochasticRungeKuttaStepperPtr.hpp:65)
        const double U1 = noise_at(a, q, 0, z0, z1), U2 = noise_at(a, q, 1, z0, z1);
        const double sdt = a.sdt;
        const double dW = dmul(U1, sdt);
        const double dZ = dmul(dmul(dmul(0.5, dt), sdt), dadd(U1, ddiv_by(U2, kSqrt3, kRcpSqrt3)));
        const double D = sc.D;
        const double s2D = sc.s2D;
        const double dtdt_x = dmul(dmul(dmul(0.5, dadd(dmul(d2, d1), dmul(D, d0))), dt), dt);
        const double xs = dadd(a.x[q], dsub(dsub(dmul(d0, dt), dmul(dmul(s2D, d1), dZ)), dtdt_x));
        const double dtdt_y = dmul(dmul(dmul(0.5, dsub(dmul(d2, d0), dmul(D, d1))), dt), dt);
        const double ys = dadd(a.y[q], dadd(dadd(dmul(d1, dt), dmul(dmul(s2D, d0), dZ)), dtdt_y));
        const double drift = sd.is_vortex ? dmul(dadd(a.omega[q], d2), dt) : dmul(d2, dt);
        const double ps = dadd(a.phi[q], dadd(dadd(dadd(drift, dmul(s2D, dW)), dmul(A0, dZ)),
                                              dmul(dmul(dmul(0.5, A1), dt), dt)));
        a.x[q] = wrap_1d(xs, sc.rL, sc.L);
        a.y[q] = wrap_1d(ys, sc.rL, sc.L);
        a.phi[q] = ps;
      }
    }
  } else {
    // FP32C: right-hand sides and increments in float, accumulated into the
    // double positions and phase.
    float f0 = 0.0f, f1 = 0.0f;
    if (draws) philox_normal2_f(sd.seed, sd.system_id, step, (uint32_t)i, f0, f1);
    auto noise_f = [&](int k) -> float {
      if (a.noise) return (float)a.noise[(size_t)q * a.noise_m + k];
      return k == 0 ? f0 : f1;
    };
    // cos / sin of the stage phase, as the gather computed them for this slot
    const float2 csp = a.cs[p];
    const float cph = csp.x, sph = csp.y;
    const float v0 = (float)sc.v0, D = (float)sc.D, dtf = (float)dt;
    const float d0 = v0 * cph, d1 = v0 * sph;
    if constexpr (KIND == kKindSin) {
      const bool has = acc.n != 0;
      const float rate = has ? (float)sc.sigma * acc.s0 / (float)acc.n : 0.0f;
      if (epi == kEpiRkK || epi == kEpiRk4Combine) {
        if (!live) return;
        const int k = a.kq_out;
        a.kx[k][q] = (double)d0;
        a.ky[k][q] = (double)d1;
        if (has) a.kphi[k][q] = (double)rate;
        if (epi == kEpiRk4Combine) {
          const float k4p = (float)a.kphi[k][q];
          const float sx_ = (float)a.kx[0][q] + 2.0f * (float)a.kx[1][q] + 2.0f * (float)a.kx[2][q] + d0;
          const float sy_ = (float)a.ky[0][q] + 2.0f * (float)a.ky[1][q] + 2.0f * (float)a.ky[2][q] + d1;
          const float sp_ = (float)a.kphi[0][q] + 2.0f * (float)a.kphi[1][q] + 2.0f * (float)a.kphi[2][q] + k4p;
          const float sixth = dtf / 6.0f;
          a.x[q] = wrap_1d(a.x[q] + (double)(sx_ * sixth), sc.rL, sc.L);
          a.y[q] = wrap_1d(a.y[q] + (double)(sy_ * sixth), sc.rL, sc.L);
          a.phi[q] = a.phi[q] + (double)(sp_ * sixth);
        }
      } else if (epi == kEpiEuler || epi == kEpiEulerPtr) {
        if (!live) return;
        const float xi = noise_f(0);
        const float sdt = sqrtf(dtf);
        const float s2D = sqrtf(2.0f * D);
        const float drift = (epi == kEpiEuler && sd.is_vortex) ? (float)a.omega[q] + rate : rate;
        a.x[q] = wrap_1d(a.x[q] + (double)(dtf * d0), sc.rL, sc.L);
        a.y[q] = wrap_1d(a.y[q] + (double)(dtf * d1), sc.rL, sc.L);
        a.phi[q] = a.phi[q] + (double)(dtf * drift + sdt * s2D * xi);
      } else if (epi == kEpiSrk1) {
        a.dphi_s[p] = (double)rate;
        a.dphi_f[p] = rate;
        a.cnt_s[p] = acc.n;
      }
    } else {
      const float inv_n = acc.n ? 1.0f / (float)acc.n : 0.0f;
      const float s2D = sqrtf(2.0f * D);
      const float A0 = (acc.s0 * inv_n) * (-s2D);
      const float A1 = acc.s1 * inv_n + (-2.0f * D) * il.dphif;
      const float d2 = il.dphif;
      if (epi == kEpiSrk2Out) {
        a.out_d[3 * (size_t)q] = (double)d0;
        a.out_d[3 * (size_t)q + 1] = (double)d1;
        a.out_d[3 * (size_t)q + 2] = (double)d2;
        a.out_a[2 * (size_t)q] = (double)A0;
        a.out_a[2 * (size_t)q + 1] = (double)A1;
      } else {
        if (!live) return;
        const float U1 = noise_f(0), U2 = noise_f(1);
        const float sdt = sqrtf(dtf);
        const float dW = U1 * sdt;
        const float dZ = 0.5f * dtf * sdt * (U1 + U2 * 0.57735026918962576f);
        const float dx = d0 * dtf - s2D * d1 * dZ - 0.5f * (d2 * d1 + D * d0) * dtf * dtf;
        const float dy = d1 * dtf + s2D * d0 * dZ + 0.5f * (d2 * d0 - D * d1) * dtf * dtf;
        const float drift = (sd.is_vortex ? (float)a.omega[q] + d2 : d2) * dtf;
        const float dp = drift + s2D * dW + A0 * dZ + 0.5f * A1 * dtf * dtf;
        a.x[q] = wrap_1d(a.x[q] + (double)dx, sc.rL, sc.L);
        a.y[q] = wrap_1d(a.y[q] + (double)dy, sc.rL, sc.L);
        a.phi[q] = a.phi[q] + (double)dp;
      }
    }
  }
}

template <int PREC, int KIND>
__device__ __forceinline__ void load_i(const KArgs &a, const SysConst &sc, ILane &il, int p, bool valid) {
  il.p = p;
  il.valid = valid;
  if (!valid) return;
  il.x = a.sx[p];
  il.y = a.sy[p];
  il.phi = a.sphi[p];
  if (!sc.allpairs) {
    const float2 f = a.fxy[p];
    il.fx = f.x;
    il.fy = f.y;
  }
  if constexpr (PREC == kPrecFP32C) {
    // cos / sin of (phi + alpha) from the stage phase's cos / sin (made by the
    // gather) by the angle-addition identity
    const float2 t = a.cs[p];
    il.ca = t.x * sc.cos_a - t.y * sc.sin_a;
    il.sa = t.y * sc.cos_a + t.x * sc.sin_a;
  }
  if constexpr (KIND == kKindCos2) {
    il.card = (double)a.cnt_s[p];
    il.rcard = drcp(il.card);  // unused (and infinite) when n_i = 0: no pairs
    il.dphi = a.dphi_s[p];
    if constexpr (PREC == kPrecFP32C) il.dphif = a.dphi_f[p];
  } else {
    il.dphi = 0.0;
    il.dphif = 0.0f;
  }
}

// FP32X: one particle's exact neighbour sums.  Pass 1 (kKindSin): c, s =
// sum_j cos phi_j, sum_j sin phi_j; pass 2 (kKindCos2): the same weighted by
// the neighbours' pass-1 phase rates d_j.  The integer sums over all staging
// rounds are converted to double once (from_fixed128).
struct XSums {
  double c, s;
  int n;
};

// FP32X epilogue: the sums become the plain form's accumulators by the
// angle-addition identities (theta_i = phi_i + alpha):
//   sum_j sin(phi_j - theta_i) = cos(theta_i) sum sin phi_j - sin(theta_i) sum cos phi_j
//   sum_j cos(phi_j - theta_i) = cos(theta_i) sum cos phi_j + sin(theta_i) sum sin phi_j
// and the FP64 epilogue finishes the step with the plain form's formulas and
// normals.  The SRK second pass's per-term divisions by n_i
// (ChimeraSystem.cpp:634-637) become one division of each sum.
template <int KIND>
__device__ void epilogue_fp32x(const KArgs &a, int epi, const SysDesc &sd, const ILane &il, const XSums &x,
                               int q) {
  const SysConst &sc = sd.sc;
  const int p = il.p;
  const longlong2 cq = a.ics[p];
  const double2 cs = make_double2(from_fixed(cq.x, kXQ), from_fixed(cq.y, kXQ));
  const double ct = dsub(dmul(cs.x, sc.cos_ad), dmul(cs.y, sc.sin_ad));  // cos(phi_i + alpha)
  const double st = dadd(dmul(cs.y, sc.cos_ad), dmul(cs.x, sc.sin_ad));  // sin(phi_i + alpha)
  Acc<kPrecFP64> acc;
  acc.n = x.n;
  acc.s1 = 0.0;
  if constexpr (KIND == kKindSin) {
    acc.s0 = x.n ? dsub(dmul(x.s, ct), dmul(x.c, st)) : 0.0;
    if (epi == kEpiSrk1) {
      // what the second pass needs: this particle's sum of cosines and its
      // rate (the FP64 epilogue's value) times cos phi_i, sin phi_i
      const double rate = x.n ? ddiv(dmul(sc.sigma, acc.s0), (double)x.n) : 0.0;
      a.scos[p] = x.n ? dadd(dmul(x.c, ct), dmul(x.s, st)) : 0.0;
      a.iws[p] = make_longlong2(to_fixed(dmul(rate, cs.x), sc.xq2), to_fixed(dmul(rate, cs.y), sc.xq2));
    }
  } else {
    const double scs = a.scos[p];
    if (x.n) {
      const double n = (double)x.n;
      acc.s0 = ddiv(scs, n);
      // sum_j (d_j - d_i) cos(phi_j - theta_i) / n_i
      acc.s1 = ddiv(dsub(dadd(dmul(x.c, ct), dmul(x.s, st)), dmul(il.dphi, scs)), n);
    } else {
      acc.s0 = 0.0;
    }
  }
  epilogue<kPrecFP64, KIND>(a, epi, sd, il, acc, q, &cs);
}

// FP32X epilogues as their own dense launch: one thread per cell-order slot,
// so the FP64 per-particle work (rates, noise, the stepper update) runs on
// full warps, while the neighbour kernels, whose warps cover cells of a few
// particles, only write each particle's sums (xsum, xcnt).  All-pairs systems
// finish in their own (FP64) kernel.
template <int KIND>
__global__ void __launch_bounds__(256) k_epilogue_fp32x(KArgs a, int epi) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n_active) return;
  const SysDesc &sd = a.sys[a.sys_of_c[cell_of_slot(a, p)]];
  const SysConst &sc = sd.sc;
  if (sc.allpairs) return;
  ILane il;
  load_i<kPrecFP32X, KIND>(a, sc, il, p, true);
  const double2 v = a.xsum[p];
  const XSums x{v.x, v.y, a.xcnt[p]};
  epilogue_fp32x<KIND>(a, epi, sd, il, x, a.pidx[p]);
}

constexpr int kPassWarps = 4;
constexpr int kPassThreads = kPassWarps * kWarp;
constexpr int kIPL = 2;  // i particles per lane: a warp covers a 64-particle cell tile

// Neighbour diagnostics (counts, lists in visiting order, local order
// parameter): one warp per cell tile, two particles per lane, the 9 stencil
// cells in the reference's order (ChimeraSystem.cpp:39-44) and within each the
// members in ascending index, 32 candidates at a time through shared memory.
// Decisions as everywhere: float prefilter, the reference's FP64 test near the
// cutoff.
template <int PREC, int KIND>
__global__ void __launch_bounds__(kPassThreads) k_cell_pass(KArgs a, int epi) {
  __shared__ float4 stage[kPassWarps][kWarp];
  const int w = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const int gwarp = blockIdx.x * kPassWarps + w;
  const int nwarps = gridDim.x * kPassWarps;
  for (int c = gwarp; c < a.ncell_total; c += nwarps) {
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    if (sc.allpairs) continue;
    const int nc = sc.nc;
    const bool exact_all = sc.exact_all != 0;
    const int cb = a.cell_start[c], ce = a.cell_start[c + 1];
    const int cl = c - sd.c0, cx = cl % nc, cy = cl / nc;
    for (int base = cb; base < ce; base += kIPL * kWarp) {
      ILane il[kIPL];
      Acc<PREC> acc[kIPL];
      long long wpos[kIPL];
#pragma unroll
      for (int k = 0; k < kIPL; ++k) {
        const int p = base + k * kWarp + lane;
        load_i<PREC, KIND>(a, sc, il[k], p, p < ce);
        acc[k].init();
        wpos[k] = (a.list_idx && il[k].valid) ? a.list_off[a.pidx[p]] : 0;
      }
      for (int q = 0; q < 9; ++q) {
        const int ox = (q % 3) - 1, oy = (q / 3) - 1;  // {-1,-1},{0,-1},{1,-1},{-1,0},...
        const int cj = sd.c0 + adjust_cell(cy + oy, nc) * nc + adjust_cell(cx + ox, nc);
        const int ja = a.cell_start[cj], jb = a.cell_start[cj + 1];
        const float shx = (float)ox * sc.cell_f, shy = (float)oy * sc.cell_f;
        for (int jbase = ja; jbase < jb; jbase += kWarp) {
          const int pl = jbase + lane;
          __syncwarp();
          if (pl < jb) {
            const float2 f = a.fxy[pl];
            stage[w][lane] = make_float4(f.x + shx, f.y + shy, 0.0f, 0.0f);
          }
          __syncwarp();
          const int cnt = min(kWarp, jb - jbase);
          for (int t = 0; t < cnt; ++t) {
            const float4 cj4 = stage[w][t];
            const int pj = jbase + t;
#pragma unroll
            for (int k = 0; k < kIPL; ++k) {
              if (!il[k].valid || pj == il[k].p) continue;
              const float dx = cj4.x - il[k].fx, dy = cj4.y - il[k].fy;
              const float d2 = dx * dx + dy * dy;
              if (exact_all || d2 <= sc.hi2) {
                const bool in = (!exact_all && d2 < sc.lo2) ||
                                exact_within(sc, il[k].x, il[k].y, a.sx[pj], a.sy[pj]);
                if (in) accept_pair<PREC, KIND>(a, sd, il[k], acc[k], pj, 0.0f, 0.0f, 0.0f, wpos[k]);
              }
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kIPL; ++k)
        if (il[k].valid) epilogue<PREC, KIND>(a, epi, sd, il[k], acc[k], a.pidx[il[k].p]);
    }
  }
}

// All pairs (rho > L/4): ChimeraSystem.cpp:117-255.  An all-pairs system's
// particles form one cell, in index order.  A work item is one block of T
// particles of one such system, so a large system spreads over many CTAs;
// one thread per i walks j ascending (the reference's order), with the exact
// FP64 test on unwrapped stage positions.  T is the CTA width: 128, or 32
// (one warp per CTA, four times the CTAs) when the all-pairs systems hold too
// few particles to give every SM work at 128 (each thread's sums are the
// same either way).
constexpr int kAllPairsThreads = 128;
constexpr int kAllPairsThreadsSmall = 32;

template <int PREC, int KIND, int T = kAllPairsThreads>
__global__ void __launch_bounds__(T) k_allpairs_pass(KArgs a, int epi) {
  __shared__ double tx[T], ty[T];
  __shared__ float2 tcs[T];
  __shared__ float td[T];
  for (int item = blockIdx.x;; item += gridDim.x) {
    // the item's system (w) and particle block (rest), uniform over the CTA
    int w = 0, rest = item, cb = 0, ce = 0;
    for (; w < a.n_ap; ++w) {
      const int cw = a.ap_cells[w];
      cb = a.cell_start[cw];
      ce = a.cell_start[cw + 1];
      const int nb = (ce - cb + T - 1) / T;
      if (rest < nb) break;
      rest -= nb;
    }
    if (w >= a.n_ap) break;
    const int c = a.ap_cells[w];
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    {
      const int ib = cb + rest * T;
      const int i = ib + threadIdx.x;
      ILane il;
      Acc<PREC> acc;
      load_i<PREC, KIND>(a, sc, il, i, i < ce);
      acc.init();
      long long wpos = (a.list_idx && il.valid) ? a.list_off[a.pidx[i]] : 0;
      for (int jt = cb; jt < ce; jt += T) {
        const int jl = jt + threadIdx.x;
        __syncthreads();
        if (jl < ce) {
          tx[threadIdx.x] = a.sx[jl];
          ty[threadIdx.x] = a.sy[jl];
          if constexpr (PREC == kPrecFP32C) {
            tcs[threadIdx.x] = a.cs[jl];
            if constexpr (KIND == kKindCos2) td[threadIdx.x] = a.dphi_f[jl];
          }
        }
        __syncthreads();
        const int cnt = min(T, ce - jt);
        if (!il.valid) continue;
        for (int t = 0; t < cnt; ++t) {
          const int j = jt + t;
          if (j == i) continue;
          if (exact_within(sc, il.x, il.y, tx[t], ty[t])) {
            float cc = 0.0f, ss = 0.0f, dj = 0.0f;
            if constexpr (PREC == kPrecFP32C) {
              cc = tcs[t].x;
              ss = tcs[t].y;
              if constexpr (KIND == kKindCos2) dj = td[t];
            }
            accept_pair<PREC, KIND>(a, sd, il, acc, j, cc, ss, dj, wpos);
          }
        }
      }
      if (il.valid) epilogue<PREC, KIND>(a, epi, sd, il, acc, a.pidx[i]);
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Per-call step bookkeeping of every system: the call takes
// budget = min(nsteps, remaining) steps, after which the system is frozen.
__global__ void k_begin_call(SysDesc *sys, int nsys, int nsteps) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const long long r = sys[s].remaining;
  sys[s].budget = (int)(r < (long long)nsteps ? (r > 0 ? r : 0) : nsteps);
}

__global__ void k_end_call(SysDesc *sys, int nsys) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  sys[s].step += (unsigned long long)sys[s].budget;
  sys[s].remaining -= sys[s].budget;
  sys[s].budget = 0;
}

// dense index -> system, and global cell -> system, from the layout tables
__global__ void k_layout_maps(const SysDesc *sys, int nsys, int n_active, int ncell_total,
                              int *sys_of_p, int *sys_of_c) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n_active) {
    int lo = 0, hi = nsys - 1;  // last system with dense_p0 <= g
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (sys[mid].dense_p0 <= g) lo = mid; else hi = mid - 1;
    }
    sys_of_p[g] = lo;
  }
  if (g < ncell_total) {
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (sys[mid].c0 <= g) lo = mid; else hi = mid - 1;
    }
    sys_of_c[g] = lo;
  }
}

__global__ void k_aos_to_soa(const double *__restrict__ aos, int n, double *x, double *y,
                             double *phi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = aos[3 * (size_t)i];
  y[i] = aos[3 * (size_t)i + 1];
  phi[i] = aos[3 * (size_t)i + 2];
}

__global__ void k_soa_to_aos(const double *x, const double *y, const double *phi, int n,
                             double *__restrict__ aos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  aos[3 * (size_t)i] = x[i];
  aos[3 * (size_t)i + 1] = y[i];
  aos[3 * (size_t)i + 2] = phi[i];
}

// Philox normals of steps [first, first + nsteps) in the injection layout.
__global__ void k_export_noise(uint64_t seed, uint32_t system_id, uint64_t first, int nsteps,
                               int n, int m, double *out) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (long long)nsteps * n) return;
  const int s = (int)(g / n), i = (int)(g % n);
  double z0, z1;
  philox_normal2(seed, system_id, first + (uint64_t)s, (uint32_t)i, z0, z1);
  double *o = out + ((size_t)s * n + i) * m;
  o[0] = z0;
  if (m > 1) o[1] = z1;
}

// a[i] / b[i] as ddiv and as ddiv_by with the reciprocal; counts the pairs
// whose results differ in any bit (spc_check_division).
__global__ void k_check_division(long long n, const double *__restrict__ a, const double *__restrict__ b,
                                 unsigned long long *bad) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double x = a[i], d = b[i];
    const double q0 = ddiv(x, d), q1 = ddiv_by(x, d, drcp(d));
    if (__double_as_longlong(q0) != __double_as_longlong(q1)) atomicAdd(bad, 1ull);
  }
}

// sin and cos of x[i] from separate launches (nothing to merge) and from one
// sincos, for spc_check_sincos.
__global__ void k_sin_only(long long n, const double *__restrict__ x, double *__restrict__ s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s[i] = sin(x[i]);
}
__global__ void k_cos_only(long long n, const double *__restrict__ x, double *__restrict__ c) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    c[i] = cos(x[i]);
}
__global__ void k_sincos_cmp(long long n, const double *__restrict__ x, const double *__restrict__ s,
                             const double *__restrict__ c, unsigned long long *bad) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double sn, cn;
    sincos(x[i], &sn, &cn);
    if (__double_as_longlong(sn) != __double_as_longlong(s[i]) ||
        __double_as_longlong(cn) != __double_as_longlong(c[i]))
      atomicAdd(bad, 1ull);
  }
}

__global__ void k_philox_kat(U4 c, uint32_t k0, uint32_t k1, uint32_t *out) {
  const U4 o = philox4x32_10(c, k0, k1);
  out[0] = o.x;
  out[1] = o.y;
  out[2] = o.z;
  out[3] = o.w;
}

// Global order parameter partial sums (FP64) of phi[0..n): sum cos, sum sin.
__global__ void k_order_sum(const double *phi, int n, double *out2) {
  __shared__ double sc_[256], ss_[256];
  double c = 0.0, s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    c += cos(phi[i]);
    s += sin(phi[i]);
  }
  sc_[threadIdx.x] = c;
  ss_[threadIdx.x] = s;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      sc_[threadIdx.x] += sc_[threadIdx.x + off];
      ss_[threadIdx.x] += ss_[threadIdx.x + off];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out2[2 * blockIdx.x] = sc_[0];
    out2[2 * blockIdx.x + 1] = ss_[0];
  }
}

}  // namespace spc
