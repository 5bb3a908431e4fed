// Host-side engine behind both C-ABI object kinds (a single-system handle is
// an engine holding one system; a batch holds many).
//
// An engine owns, on one CUDA stream:
//  * a particle pool for the state of every admitted system (x, y, phi,
//    omega, and RK4's persistent stage rates), first-fit allocated per system;
//  * per-evaluation scratch sized to the pool (stage arrays, sort buffers,
//    cell-order copies, float prefilter data, FP32C neighbour bitmasks) and to
//    the cell capacity (cell table, cell -> system map);
//  * the device table of active systems (SysDesc) and its host mirror.
// Admitting or releasing a system changes the layout (dense order of the
// active systems' particles and their global cell ranges); the next step
// rebuilds the device tables and drops any cached CUDA graph.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/spc_gb300.h"
#include "spc_kernels.cuh"
#include "spc_sort.cuh"
#include "spc_tile.cuh"
#include "spc_warp.cuh"
#include "spc_verlet.cuh"
#include "spc_va.cuh"

namespace spc {

inline std::mutex &err_mutex() {
  static std::mutex m;
  return m;
}
inline std::string &global_error() {
  static std::string s;
  return s;
}

// A positive finite power of two (then x / L equals x * (1 / L) exactly).
inline int is_pow2(double L) {
  int e = 0;
  return std::frexp(L, &e) == 0.5 ? 1 : 0;
}

inline int blocks_for(long long n, int threads) { return (int)((n + threads - 1) / threads); }

inline int noise_per_particle(int stepper) {
  switch (stepper) {
    case SPC_STEPPER_SRK: return 2;
    case SPC_STEPPER_RK4: return 0;
    default: return 1;
  }
}

// Per-system constants from the public parameters (ChimeraSystem.cpp:19-33).
inline SysConst make_sysconst(const spc_params &p, int n) {
  SysConst sc{};
  sc.n = n;
  sc.L = p.L;
  sc.rL = 1.0 / p.L;
  sc.rho = p.rho;
  sc.rho2 = p.rho * p.rho;
  sc.v0 = p.v0;
  sc.sigma = p.sigma;
  sc.alpha = p.alpha;
  sc.D = p.D_phi;
  sc.allpairs = !(p.rho <= 0.25 * p.L);
  sc.nc = sc.allpairs ? 1 : std::max(1, (int)(p.L / p.rho));
  sc.ncell = sc.nc * sc.nc;
  sc.cell = p.L / sc.nc;
  sc.cell_f = (float)sc.cell;
  // prefilter band: a relative 3e-5 of rho^2 on each side, far wider than the
  // float error of the cell-relative dr^2 (about 3e-6 rho^2 for cells <= 4/3 rho)
  sc.lo2 = (float)(sc.rho2 * (1.0 - 3e-5));
  sc.hi2 = (float)(sc.rho2 * (1.0 + 3e-5));
  sc.exact_all = (p.flags & SPC_FLAG_EXACT_ALL) ? 1 : 0;
  sc.L_pow2 = is_pow2(p.L);
  sc.cos_a = (float)std::cos(p.alpha);
  sc.sin_a = (float)std::sin(p.alpha);
  sc.s2D = std::sqrt(2.0 * p.D_phi);  // correctly rounded, as the device's sqrt
  sc.cos_ad = std::cos(p.alpha);
  sc.sin_ad = std::sin(p.alpha);
  {
    // |phase rate| <= |sigma| (sigma times a mean of sines): 2^e >= |sigma|
    int e = 0;
    while (e < 40 && std::ldexp(1.0, e) < std::fabs(p.sigma)) ++e;
    sc.xq2 = kXQ - e - 1;  // one more bit of headroom for the rate's rounding
  }
  if (p.model == SPC_MODEL_VORTEX_ARRAYS) {
    sc.va = 1;
    sc.mu_plus = p.mu_plus;
    sc.mu_minus = p.mu_minus;
    sc.xi_a = p.xi_a;
    sc.xi_r = p.xi_r;
    sc.kappa = p.kappa;
    const double rm = std::max(p.rho, p.xi_r);
    sc.va_r2 = (float)(rm * rm * (1.0 + 3e-5));
    // IEEE double arithmetic on the host: the same roundings as the device's
    sc.va_w = p.rho - p.xi_a;
    sc.va_xa2 = p.xi_a * p.xi_a;
    sc.va_rw = 1.0 / sc.va_w;
    sc.va_rxa = 1.0 / p.xi_a;
    sc.va_rxa2 = 1.0 / sc.va_xa2;
  }
  // Verlet rows over a (2R+1)^2 stencil of rho-cells; needs 2R+1 distinct cells
  if (p.neighbour == SPC_NEIGHBOUR_VERLET && !sc.allpairs && !sc.va) {
    const double rmax = p.rho + p.skin;
    const int R = (int)std::ceil(rmax / sc.cell);
    if (R >= 1 && R <= kVMaxR && sc.nc >= 2 * R + 1) {
      sc.vR = R;
      sc.vr2 = (float)(rmax * rmax * (1.0 + 1e-4));
      const double h = 0.5 * p.skin * (1.0 - 1e-6);
      sc.vdisp2 = h * h;
    }
  }
  return sc;
}

inline int validate_params(const spc_params *p, int n, std::string &why) {
  char buf[256];
  auto bad = [&](const char *m) {
    why = m;
    return SPC_ERR_INVALID;
  };
  if (!p) return bad("params is NULL");
  if (n <= 0) {
    snprintf(buf, sizeof(buf), "n must be positive (got %d)", n);
    return bad(buf);
  }
  if (!(p->L > 0.0) || !std::isfinite(p->L)) return bad("L must be positive");
  if (!(p->rho > 0.0) || !std::isfinite(p->rho)) return bad("rho must be positive");
  if (!(p->D_phi >= 0.0) || !std::isfinite(p->D_phi)) return bad("D_phi must be >= 0");
  if (!std::isfinite(p->v0) || !std::isfinite(p->sigma) || !std::isfinite(p->alpha))
    return bad("v0, sigma, alpha must be finite");
  if (p->model != SPC_MODEL_CHIMERA && p->model != SPC_MODEL_VORTEX && p->model != SPC_MODEL_VORTEX_ARRAYS)
    return bad("unknown model");
  if (p->model == SPC_MODEL_VORTEX_ARRAYS) {
    if (p->precision != SPC_PRECISION_FP64) return bad("the vortex-arrays model runs in plain FP64");
    if (p->stepper == SPC_STEPPER_EULER)
      return bad("the vortex-arrays model pairs with the Euler-Ptr, SRK and RK4 steppers");
    if (!(p->xi_a > 0.0) || !std::isfinite(p->xi_a) || !(p->xi_r >= 0.0) || !std::isfinite(p->xi_r) ||
        !std::isfinite(p->mu_plus) || !std::isfinite(p->mu_minus) || !std::isfinite(p->kappa))
      return bad("vortex arrays: xi_a > 0, xi_r >= 0, finite mu and kappa");
  }
  if (p->stepper < SPC_STEPPER_EULER || p->stepper > SPC_STEPPER_EULER_PTR) return bad("unknown stepper");
  if (p->model == SPC_MODEL_VORTEX && p->stepper != SPC_STEPPER_SRK && p->stepper != SPC_STEPPER_EULER)
    return bad("the vortex model's natural frequencies enter the Euler and stochastic Runge-Kutta drifts only");
  if (p->neighbour != SPC_NEIGHBOUR_CELL && p->neighbour != SPC_NEIGHBOUR_VERLET)
    return bad("unknown neighbour search");
  if (p->precision != SPC_PRECISION_FP64 && p->precision != SPC_PRECISION_FP32C &&
      p->precision != SPC_PRECISION_FP32X)
    return bad("unknown precision");
  if (p->precision == SPC_PRECISION_FP32X && p->neighbour == SPC_NEIGHBOUR_VERLET)
    return bad("the FP32X form runs the cell list (Verlet rows are built for FP64 and FP32C)");
  if (p->neighbour == SPC_NEIGHBOUR_VERLET && !(p->skin > 0.0)) return bad("Verlet skin must be positive");
  if (p->rho <= 0.25 * p->L && std::floor(p->L / p->rho) > 46340.0) return bad("too many cells");
  return SPC_OK;
}

struct SysHost {
  bool used = false;
  spc_params p{};
  int n = 0;
  int pool_p0 = 0;
  int ncell = 0;  // cells it occupies in the global cell list (1 for all pairs)
  SysConst sc{};
  unsigned long long step = 0;
  long long remaining = 0;
  bool omega_set = false;
};

struct Engine {
  int stepper = 0, precision = 0, device = 0;
  cudaStream_t stream = nullptr;
  // cell units: the units kernel runs on `side`, forked from and joined back
  // to `stream`, beside the cell-tile kernel (float forms)
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  std::vector<void *> allocs;
  std::string err;
  // capacities
  int pool_cap = 0, sys_cap = 0, cell_cap = 0, tile_cap = 0;
  KArgs a{};
  SysDesc *d_sys = nullptr;
  int *d_ap = nullptr;      // cells of the all-pairs systems the all-pairs kernel integrates
  int *d_ap_all = nullptr;  // ... and of every all-pairs system (diagnostics)
  int n_ap_all = 0;
  // particle blocks (work items of k_allpairs_pass) of those systems, in
  // blocks of kAllPairsThreads and of kAllPairsThreadsSmall particles
  int ap_items = 0, ap_items_all = 0;
  int ap_items_small = 0, ap_items_all_small = 0;
  unsigned long long *d_clamped = nullptr;
  uint32_t *keys_alt = nullptr, *vals_alt = nullptr, *hist = nullptr, *part = nullptr;
  double *aos = nullptr;  // AoS staging (12 x pool_cap doubles)
  double *order_part = nullptr;
  int order_blocks = 0;
  // host mirror
  std::vector<SysHost> slots;
  std::vector<int> order;  // active slots in layout order
  std::vector<std::pair<int, int>> free_ranges;  // (start, length), sorted by start
  int cells_used = 0;
  bool dirty = true;
  // current layout
  int nsys = 0, n_active = 0, ncell_total = 0, ntiles = 0, radix_bits = 1, sort_passes = 1;
  int ncell_tile = 0, ncell_warp = 0, ncell_va = 0;  // cells of the tile, warp and vortex-arrays systems
  bool has_cells = false;
  // tuning: cell-list systems with fewer than sparse_below particles per cell
  // (on average) run the warp-per-cell passes
  double sparse_below = kSparseBelowDefault;
  // tuning: CTAs per cell of the cell-tile kernels (0: chosen per layout)
  int tile_split_tune = 0;
  // tuning: the cells of the float cell-tile passes run as units (1) or as
  // whole groups (0)
  int cell_units_tune = 0;
  // tuning: the float cell-tile passes bin into half-cell sub-cells and run
  // every cell of at most kSplitRounds rounds as units of its halves (1)
  int subcells_tune = 0;
  // the cell-unit and sub-cell buffers (float forms; allocated at init)
  int2 *units_buf = nullptr;
  int *cell_mid_buf = nullptr;
  uint8_t *cell_near_buf = nullptr;
  std::vector<int> slot_layout;  // slot -> layout index (-1 if inactive)
  // noise injection (single-system handles)
  double *d_noise = nullptr;
  long long noise_count = 0, noise_cursor = 0;
  bool injecting = false;
  bool scratch_k = false;
  // graph cache
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  size_t graph_nodes = 0;  // kernel and memset nodes of the cached graph
  double graph_dt = 0.0;
  // profiling marks
  cudaEvent_t prof_ev[8] = {};
  bool profiling = false;
  // an engine that is a view over caller-provided memory owns nothing
  bool view = false;
  // Verlet rows (single-system handles whose parameters ask for them)
  bool verlet = false;
  bool verlet_stale = true;  // the build tables are not valid: force a build
  int vcap_alloc = 0;        // row capacity allocated
  uint16_t *vrows = nullptr;
  int *vrowlen = nullptr, *vsys = nullptr, *vcell = nullptr, *vflags = nullptr;
  double *vxb = nullptr, *vyb = nullptr;
  unsigned long long *vrebuilds = nullptr;
  // observed run loop (spc_run): two snapshot rings (device and pinned host),
  // a copy stream, and one captured chunk graph per ring
  struct RunPipe {
    cudaStream_t copy = nullptr;
    cudaEvent_t computed[2] = {}, copied[2] = {};
    double *d_ring[2] = {}, *h_ring[2] = {};
    size_t ring_doubles = 0;
    cudaGraphExec_t graph[2] = {};
    size_t graph_nodes = 0;
    int steps = 0;
    double dt = 0.0;
    std::vector<uint8_t> pattern;  // observe after chunk step s (0-based) iff pattern[s]
  } run;
};

inline int fail(Engine *e, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (e) e->err = buf;
  std::lock_guard<std::mutex> lk(err_mutex());
  global_error() = buf;
  return code;
}

#define SPC_CUDA(e, call)                                                                    \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return ::spc::fail((e), e_ == cudaErrorMemoryAllocation ? SPC_ERR_NOMEM : SPC_ERR_CUDA, \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

#define SPC_LAUNCHED(e) SPC_CUDA(e, cudaGetLastError())

#define SPC_TRY(expr)              \
  do {                             \
    int rc_ = (expr);              \
    if (rc_ != SPC_OK) return rc_; \
  } while (0)

template <class T>
int dalloc(Engine *e, T **ptr, size_t count) {
  void *p = nullptr;
  cudaError_t ce = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
  if (ce != cudaSuccess)
    return fail(e, SPC_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(ce));
  e->allocs.push_back(p);
  *ptr = (T *)p;
  return SPC_OK;
}

// The 11-bit scatter needs more than the default 48 KB of dynamic shared
// memory; the attribute is set with the device current (not a stream
// operation, so never inside a capture).
inline cudaError_t set_kernel_attributes() {
  cudaError_t ce = cudaFuncSetAttribute(k_radix_scatter<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)scatter_smem_bytes(11));
  if (ce == cudaSuccess)
    ce = cudaFuncSetAttribute(k_radix_scatter<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)scatter_smem_bytes(11));
  return ce;
}

inline int engine_set_device(Engine *e) {
  SPC_CUDA(e, cudaSetDevice(e->device));
  return SPC_OK;
}

// Bytes of device memory per pool particle and per cell for a stepper/precision.
inline void engine_footprint(int stepper, int precision, long long *per_particle, long long *per_cell) {
  long long b = 4 * 8;                       // x, y, phi, omega
  if (stepper == SPC_STEPPER_RK4) b += 12 * 8;  // k1..k4
  b += 3 * 8 + 4 * 4 + 3 * 8 + 8 + 4 + 8 + 4 + 4 + 4;  // stage, sort, cell order, fxy, pidx, dphi, cnt, sys_of_p
  if (precision == SPC_PRECISION_FP32C) b += 8 + 4 + (long long)kMaskWords * 4;  // cs, dphi_f, masks
  if (precision == SPC_PRECISION_FP32X)
    b += 16 + 16 + 8 + 16 + 4 + (long long)kMaskWords * 4;  // ics, iws, scos, xsum, xcnt, masks
  if (precision != SPC_PRECISION_FP64)  // cell units: round sums, counts, chunk counters, list
    b += kSplitRounds * ((precision == SPC_PRECISION_FP32X ? 16 : 8) + 4) + 4 + kSplitRounds * 8 / 32;
  if (precision == SPC_PRECISION_FP64) b += 8 + 8 + 4;                          // vortex-arrays outputs
  b += 12 * 8 + 4 + 4;                       // AoS staging, histogram share
  *per_particle = b;
  // cell_start, sys_of_c; float forms: unit list (two halves' worth), flag, sub-cell split and flag
  *per_cell = 4 + 4 + (precision != SPC_PRECISION_FP64 ? 2 * kSplitRounds * 8 + 1 + 4 + 1 : 0);
}

inline int engine_init(Engine *e, int stepper, int precision, int pool_cap, int sys_cap, int cell_cap) {
  e->stepper = stepper;
  e->precision = precision;
  e->pool_cap = pool_cap;
  e->sys_cap = sys_cap;
  e->cell_cap = cell_cap;
  if (cudaGetDevice(&e->device) != cudaSuccess) return fail(e, SPC_ERR_CUDA, "no CUDA device");
  if (set_kernel_attributes() != cudaSuccess) return fail(e, SPC_ERR_CUDA, "cudaFuncSetAttribute failed");
  SPC_CUDA(e, cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  const size_t N = (size_t)pool_cap;
  KArgs &a = e->a;
  e->tile_cap = (int)((N + kSortTile - 1) / kSortTile);
  SPC_TRY(dalloc(e, &a.x, N));
  SPC_TRY(dalloc(e, &a.y, N));
  SPC_TRY(dalloc(e, &a.phi, N));
  double *omega = nullptr;
  SPC_TRY(dalloc(e, &omega, N));
  a.omega = omega;
  if (stepper == SPC_STEPPER_RK4)
    for (int q = 0; q < 4; ++q) {
      SPC_TRY(dalloc(e, &a.kx[q], N));
      SPC_TRY(dalloc(e, &a.ky[q], N));
      SPC_TRY(dalloc(e, &a.kphi[q], N));
    }
  SPC_TRY(dalloc(e, &a.st_x, N));
  SPC_TRY(dalloc(e, &a.st_y, N));
  SPC_TRY(dalloc(e, &a.st_phi, N));
  SPC_TRY(dalloc(e, &a.keys, N));
  SPC_TRY(dalloc(e, &a.vals, N));
  SPC_TRY(dalloc(e, &e->keys_alt, N));
  SPC_TRY(dalloc(e, &e->vals_alt, N));
  SPC_TRY(dalloc(e, &a.sx, N));
  SPC_TRY(dalloc(e, &a.sy, N));
  SPC_TRY(dalloc(e, &a.sphi, N));
  SPC_TRY(dalloc(e, &a.fxy, N));
  SPC_TRY(dalloc(e, &a.pidx, N));
  SPC_TRY(dalloc(e, &a.dphi_s, N));
  SPC_TRY(dalloc(e, &a.cnt_s, N));
  if (precision == SPC_PRECISION_FP64) {  // vortex-arrays pass-1 outputs
    SPC_TRY(dalloc(e, &a.va_vx, N));
    SPC_TRY(dalloc(e, &a.va_vy, N));
    SPC_TRY(dalloc(e, &a.va_cnt2, N));
  }
  int *sys_of_p = nullptr, *sys_of_c = nullptr;
  SPC_TRY(dalloc(e, &sys_of_p, N));
  a.sys_of_p = sys_of_p;
  if (precision == SPC_PRECISION_FP32C) {
    SPC_TRY(dalloc(e, &a.cs, N));
    SPC_TRY(dalloc(e, &a.dphi_f, N));
    SPC_TRY(dalloc(e, &a.nbmask, (size_t)kMaskWords * N));
    SPC_TRY(dalloc(e, &a.part_f, (size_t)kSplitRounds * N));
  }
  if (precision == SPC_PRECISION_FP32X) {
    SPC_TRY(dalloc(e, &a.ics, N));
    SPC_TRY(dalloc(e, &a.iws, N));
    SPC_TRY(dalloc(e, &a.scos, N));
    SPC_TRY(dalloc(e, &a.xsum, N));
    SPC_TRY(dalloc(e, &a.xcnt, N));
    SPC_TRY(dalloc(e, &a.nbmask, (size_t)kMaskWords * N));
    SPC_TRY(dalloc(e, &a.part_x, (size_t)kSplitRounds * N));
  }
  if (precision != SPC_PRECISION_FP64) {
    // a unit cell of n_c particles lists ceil(n_c / 32) x (at most
    // kSplitRounds) units, or with sub-cells ceil(n_0 / 32) + ceil(n_1 / 32)
    // (n_0 + n_1 = n_c) times that, so (N / 32 + 2 cells) x kSplitRounds
    // entries hold any layout
    SPC_TRY(dalloc(e, &e->units_buf, ((N + kWarp - 1) / kWarp + 2 * (size_t)cell_cap) * kSplitRounds));
    SPC_TRY(dalloc(e, &e->cell_mid_buf, (size_t)cell_cap));
    SPC_TRY(dalloc(e, &e->cell_near_buf, (size_t)cell_cap));
    SPC_TRY(dalloc(e, &a.unit_count, 1));
    SPC_TRY(dalloc(e, &a.cell_unit, (size_t)cell_cap));
    SPC_TRY(dalloc(e, &a.part_n, (size_t)kSplitRounds * N));
    SPC_TRY(dalloc(e, &a.unit_done, N));
    SPC_CUDA(e, cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking));
    SPC_CUDA(e, cudaEventCreateWithFlags(&e->fork_ev, cudaEventDisableTiming));
    SPC_CUDA(e, cudaEventCreateWithFlags(&e->join_ev, cudaEventDisableTiming));
  }
  SPC_TRY(dalloc(e, &a.cell_start, (size_t)cell_cap + 1));
  SPC_TRY(dalloc(e, &sys_of_c, (size_t)cell_cap));
  a.sys_of_c = sys_of_c;
  // radix histogram table: up to 2^11 digits per tile, plus group partials
  SPC_TRY(dalloc(e, &e->hist, (size_t)(1 << 11) * e->tile_cap));
  SPC_TRY(dalloc(e, &e->part, (size_t)(1 << 11) * ((e->tile_cap + kScanGroup - 1) / kScanGroup)));
  SPC_TRY(dalloc(e, &e->d_sys, (size_t)sys_cap));
  SPC_TRY(dalloc(e, &e->d_ap, (size_t)sys_cap));
  SPC_TRY(dalloc(e, &e->d_ap_all, (size_t)sys_cap));
  SPC_TRY(dalloc(e, &e->d_clamped, 1));
  SPC_TRY(dalloc(e, &e->aos, 12 * N));
  e->order_blocks = std::min(blocks_for((long long)N, 256), 1024);
  SPC_TRY(dalloc(e, &e->order_part, 2 * (size_t)e->order_blocks));
  a.sys = e->d_sys;
  a.ap_cells = e->d_ap;
  a.clamped = e->d_clamped;
  a.hist = e->hist;
  cudaStream_t st = e->stream;
  SPC_CUDA(e, cudaMemsetAsync(omega, 0, N * 8, st));
  SPC_CUDA(e, cudaMemsetAsync(e->hist, 0, (size_t)(1 << 11) * e->tile_cap * 4, st));
  SPC_CUDA(e, cudaMemsetAsync(e->d_clamped, 0, 8, st));
  if (a.unit_done) {
    SPC_CUDA(e, cudaMemsetAsync(a.unit_done, 0, N * 4, st));
    SPC_CUDA(e, cudaMemsetAsync(a.unit_count, 0, 4, st));
  }
  if (stepper == SPC_STEPPER_RK4)
    for (int q = 0; q < 4; ++q) {
      SPC_CUDA(e, cudaMemsetAsync(a.kx[q], 0, N * 8, st));
      SPC_CUDA(e, cudaMemsetAsync(a.ky[q], 0, N * 8, st));
      SPC_CUDA(e, cudaMemsetAsync(a.kphi[q], 0, N * 8, st));
    }
  SPC_CUDA(e, cudaStreamSynchronize(st));
  e->slots.assign(sys_cap, SysHost());
  e->slot_layout.assign(sys_cap, -1);
  e->free_ranges.clear();
  e->free_ranges.push_back({0, pool_cap});
  return SPC_OK;
}

// Verlet buffers for rows of up to `cap` entries (cap <= 1024, so that the
// FP32C pass-1 bits of a row fit the 32 mask words of a particle).
// Vortex-arrays SRK single systems: room for the first pass's records of
// `cap` pairs within rho per particle (32 B each), within a budget of 4 GB;
// beyond it (or beyond cap pairs) the second pass recomputes them.
inline int engine_init_va_cache(Engine *e, int cap) {
  const size_t N = (size_t)e->pool_cap;
  cap = std::max(32, cap);
  if ((size_t)cap * N * 4 * sizeof(double) > ((size_t)4 << 30)) return SPC_OK;
  SPC_TRY(dalloc(e, &e->a.vacache, (size_t)cap * N * 4));
  e->a.vacap = cap;
  return SPC_OK;
}

// Cell-tile FP64 SRK single systems: room for the first pass's cosines of
// `cap` accepted pairs per particle (8 B each), within a budget of 4 GB;
// beyond it (or beyond cap pairs) the second pass evaluates them.
inline int engine_init_tile_cos(Engine *e, int cap) {
  const size_t N = (size_t)e->pool_cap;
  cap = std::max(32, cap);
  if ((size_t)cap * N * sizeof(double) > ((size_t)4 << 30)) return SPC_OK;
  SPC_TRY(dalloc(e, &e->a.tcos, (size_t)cap * N));
  e->a.tcap = cap;
  return SPC_OK;
}

inline int engine_init_verlet(Engine *e, int cap) {
  const size_t N = (size_t)e->pool_cap;
  cap = std::max(32, std::min(cap, kMaskWords * kWarp));
  e->verlet = true;
  e->vcap_alloc = cap;
  SPC_TRY(dalloc(e, &e->vrows, (size_t)cap * N));
  SPC_TRY(dalloc(e, &e->vrowlen, N));
  SPC_TRY(dalloc(e, &e->vsys, N));
  SPC_TRY(dalloc(e, &e->vcell, N));
  SPC_TRY(dalloc(e, &e->vxb, N));
  SPC_TRY(dalloc(e, &e->vyb, N));
  SPC_TRY(dalloc(e, &e->vflags, 2));
  SPC_TRY(dalloc(e, &e->vrebuilds, 1));
  // FP64 SRK: the first pass keeps each accepted row entry's cosine for the
  // second (sincos gives the cosine bit for bit; spc_check_sincos), within a
  // budget of 4 GB; above it the second pass evaluates the cosine itself
  double *vcos = nullptr;
  if (e->precision == SPC_PRECISION_FP64 && e->stepper == SPC_STEPPER_SRK &&
      (size_t)cap * N * sizeof(double) <= ((size_t)4 << 30))
    SPC_TRY(dalloc(e, &vcos, (size_t)cap * N));
  cudaStream_t st = e->stream;
  SPC_CUDA(e, cudaMemsetAsync(e->vrowlen, 0, N * 4, st));
  SPC_CUDA(e, cudaMemsetAsync(e->vsys, 0, N * 4, st));
  SPC_CUDA(e, cudaMemsetAsync(e->vcell, 0, N * 4, st));
  SPC_CUDA(e, cudaMemsetAsync(e->vflags, 0, 8, st));
  SPC_CUDA(e, cudaMemsetAsync(e->vrebuilds, 0, 8, st));
  SPC_CUDA(e, cudaStreamSynchronize(st));
  KArgs &a = e->a;
  a.vrows = e->vrows;
  a.vrowlen = e->vrowlen;
  a.vcap = cap;
  a.vxb = e->vxb;
  a.vyb = e->vyb;
  a.vflags = e->vflags;
  a.vrebuilds = e->vrebuilds;
  a.vcos = vcos;
  e->verlet_stale = true;
  return SPC_OK;
}

// Before enqueueing evaluations (outside any graph capture): a stale build is
// forced through the device flag that the next gather reads.
inline int verlet_prepare(Engine *e) {
  if (!e->verlet || !e->verlet_stale) return SPC_OK;
  SPC_CUDA(e, cudaMemsetAsync(e->vflags + 1, 1, 1, e->stream));
  e->verlet_stale = false;
  return SPC_OK;
}

// CTAs per cell of the cell-tile kernels: one unless tuned.  Splitting the
// 64-particle cells of a one-wave system (1024 cells) into 2-4 CTAs to even
// out the SMs' ends of pass measured 3-4% slower on GB300 (each CTA stages the
// whole stencil; the idle SM time at the end of a pass did not shrink).
inline int tile_split_for(int tune) { return tune > 0 ? tune : 1; }

inline void drop_graph(Engine *e) {
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  for (cudaGraphExec_t &g : e->run.graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

inline void engine_free(Engine *e) {
  if (!e || e->view) return;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->run.copy) cudaStreamSynchronize(e->run.copy);
  drop_graph(e);
  for (cudaEvent_t ev : e->prof_ev)
    if (ev) cudaEventDestroy(ev);
  for (int b = 0; b < 2; ++b) {
    if (e->run.computed[b]) cudaEventDestroy(e->run.computed[b]);
    if (e->run.copied[b]) cudaEventDestroy(e->run.copied[b]);
    if (e->run.h_ring[b]) cudaFreeHost(e->run.h_ring[b]);
    e->run.h_ring[b] = nullptr;
  }
  if (e->run.copy) cudaStreamDestroy(e->run.copy);
  e->run.copy = nullptr;
  if (e->side) cudaStreamSynchronize(e->side);
  if (e->fork_ev) cudaEventDestroy(e->fork_ev);
  if (e->join_ev) cudaEventDestroy(e->join_ev);
  if (e->side) cudaStreamDestroy(e->side);
  e->side = nullptr;
  e->fork_ev = e->join_ev = nullptr;
  for (void *p : e->allocs) cudaFree(p);
  e->allocs.clear();
  if (e->stream) cudaStreamDestroy(e->stream);
  e->stream = nullptr;
}

// ---------------------------------------------------------------------------
// pool allocator (first fit, coalescing)
inline int pool_take(Engine *e, int n) {
  for (size_t k = 0; k < e->free_ranges.size(); ++k) {
    auto &r = e->free_ranges[k];
    if (r.second >= n) {
      const int at = r.first;
      r.first += n;
      r.second -= n;
      if (r.second == 0) e->free_ranges.erase(e->free_ranges.begin() + k);
      return at;
    }
  }
  return -1;
}

inline void pool_give(Engine *e, int at, int n) {
  auto &fr = e->free_ranges;
  fr.push_back({at, n});
  std::sort(fr.begin(), fr.end());
  std::vector<std::pair<int, int>> merged;
  for (auto &r : fr) {
    if (!merged.empty() && merged.back().first + merged.back().second == r.first)
      merged.back().second += r.second;
    else
      merged.push_back(r);
  }
  fr.swap(merged);
}

// Admit a system: its state goes to a pool range; returns the slot.
inline int engine_admit(Engine *e, const spc_params &p, int n, long long steps, int *slot_out) {
  std::string why;
  int rc = validate_params(&p, n, why);
  if (rc) return fail(e, rc, "%s", why.c_str());
  if (p.stepper != e->stepper) return fail(e, SPC_ERR_INVALID, "stepper differs from the batch's");
  if (p.precision != e->precision) return fail(e, SPC_ERR_INVALID, "precision differs from the batch's");
  SysConst sc = make_sysconst(p, n);
  const int ncell = sc.allpairs ? 1 : sc.ncell;
  int slot = -1;
  for (int s = 0; s < e->sys_cap; ++s)
    if (!e->slots[s].used) {
      slot = s;
      break;
    }
  if (slot < 0) return fail(e, SPC_ERR_CAPACITY, "no free system slot (capacity %d)", e->sys_cap);
  if (e->cells_used + ncell > e->cell_cap)
    return fail(e, SPC_ERR_CAPACITY, "cells: %d used + %d needed > %d", e->cells_used, ncell, e->cell_cap);
  const int at = pool_take(e, n);
  if (at < 0) return fail(e, SPC_ERR_CAPACITY, "no contiguous pool range of %d particles", n);
  SysHost &h = e->slots[slot];
  h = SysHost();
  h.used = true;
  h.p = p;
  h.n = n;
  h.pool_p0 = at;
  h.ncell = ncell;
  h.sc = sc;
  h.step = 0;
  h.remaining = steps < 0 ? (1ll << 62) : steps;
  e->cells_used += ncell;
  e->order.push_back(slot);
  e->dirty = true;
  *slot_out = slot;
  return SPC_OK;
}

inline int engine_release(Engine *e, int slot) {
  if (slot < 0 || slot >= e->sys_cap || !e->slots[slot].used)
    return fail(e, SPC_ERR_INVALID, "no system in slot %d", slot);
  SysHost &h = e->slots[slot];
  pool_give(e, h.pool_p0, h.n);
  e->cells_used -= h.ncell;
  h.used = false;
  e->order.erase(std::find(e->order.begin(), e->order.end(), slot));
  e->dirty = true;
  return SPC_OK;
}

inline SysDesc desc_of(const SysHost &h, int dense_p0, int c0) {
  SysDesc d{};
  d.sc = h.sc;
  d.pool_p0 = h.pool_p0;
  d.dense_p0 = dense_p0;
  d.c0 = c0;
  d.is_vortex = h.p.model == SPC_MODEL_VORTEX;
  d.system_id = h.p.system_id;
  d.seed = h.p.seed;
  d.step = h.step;
  d.remaining = h.remaining;
  d.budget = 0;
  return d;
}

// 0: cell list, dense cells (cell-tile kernels); 1: cell list, sparse cells
// (warp-per-cell kernel); 2: vortex-arrays model (its own kernel, cell list or
// all pairs); 3: all pairs.
inline int system_class(const Engine *e, const SysHost &h) {
  if (h.sc.va) return 2;
  if (h.sc.allpairs) return 3;
  return (double)h.n < e->sparse_below * (double)h.ncell ? 1 : 0;
}

// Sub-cells are in effect: asked for, on a float form's cell-list engine.
inline bool subcells_on(const Engine *e) {
  return e->subcells_tune && e->precision != SPC_PRECISION_FP64 && !e->verlet;
}

// Rebuild the device layout tables from the host mirror.
// What a captured step graph bakes in beyond device pointers: kernel grid
// sizes and the counts passed by value.  A layout that leaves these unchanged
// (new step counters or budgets, a system replaced by one of the same shape)
// keeps the cached graphs, whose kernels read the rewritten tables.
inline std::vector<long long> launch_shape(const Engine *e) {
  const KArgs &a = e->a;
  return {e->nsys, e->n_active, e->ncell_total, e->ntiles, e->radix_bits, e->sort_passes, e->ncell_tile,
          e->ncell_warp, e->ncell_va, e->n_ap_all, e->has_cells, a.n_ap, a.tile_split, a.hist_len,
          e->ap_items, e->ap_items_all, e->ap_items_small, e->ap_items_all_small, a.units != nullptr,
          a.cell_mid != nullptr};
}

inline int engine_layout(Engine *e) {
  if (!e->dirty) return SPC_OK;
  const std::vector<long long> shape0 = launch_shape(e);
  e->verlet_stale = true;  // slots and systems move: rebuild the rows
  std::vector<SysDesc> table;
  std::vector<int> ap, ap_all;
  int dense = 0, cells = 0;
  std::fill(e->slot_layout.begin(), e->slot_layout.end(), -1);
  // cell-tile systems first, then warp-per-cell, vortex-arrays and all-pairs
  // systems, so that each neighbour kernel covers one contiguous range of cells
  int ncell_tile = 0, ncell_warp = 0, ncell_va = 0;
  e->ap_items = e->ap_items_all = 0;
  e->ap_items_small = e->ap_items_all_small = 0;
  for (int cls = 0; cls < 4; ++cls) {
    for (int slot : e->order) {
      const SysHost &h = e->slots[slot];
      if (system_class(e, h) != cls) continue;
      e->slot_layout[slot] = (int)table.size();
      table.push_back(desc_of(h, dense, cells));
      const int blocks = (h.n + kAllPairsThreads - 1) / kAllPairsThreads;
      const int blocks_small = (h.n + kAllPairsThreadsSmall - 1) / kAllPairsThreadsSmall;
      if (cls == 3) {
        ap.push_back(cells);
        e->ap_items += blocks;
        e->ap_items_small += blocks_small;
      }
      if (h.sc.allpairs) {
        ap_all.push_back(cells);
        e->ap_items_all += blocks;
        e->ap_items_all_small += blocks_small;
      }
      dense += h.n;
      cells += h.ncell;
      if (cls == 0) ncell_tile += h.ncell;
      if (cls == 1) ncell_warp += h.ncell;
      if (cls == 2) ncell_va += h.ncell;
    }
  }
  e->ncell_tile = ncell_tile;
  e->ncell_warp = ncell_warp;
  e->ncell_va = ncell_va;
  e->nsys = (int)table.size();
  e->n_active = dense;
  e->ncell_total = cells;
  e->ntiles = std::max(1, (dense + kSortTile - 1) / kSortTile);
  // sub-cells: two sort keys per cell
  const bool sub = subcells_on(e);
  const int nkeys = sub ? 2 * cells : cells;
  int bits = 1;
  while (bits < 31 && (1u << bits) < (unsigned)std::max(nkeys, 2)) ++bits;
  e->sort_passes = (bits + 10) / 11;
  e->radix_bits = (bits + e->sort_passes - 1) / e->sort_passes;
  e->has_cells = ncell_tile + ncell_warp > 0;
  e->n_ap_all = (int)ap_all.size();
  KArgs &a = e->a;
  a.nsys = e->nsys;
  a.n_active = e->n_active;
  a.ncell_total = e->ncell_total;
  a.ncell_tile = e->ncell_tile;
  a.tile_split = tile_split_for(e->tile_split_tune);
  a.units = (e->cell_units_tune || sub) ? e->units_buf : nullptr;
  a.cell_mid = sub ? e->cell_mid_buf : nullptr;
  a.cell_near = sub ? e->cell_near_buf : nullptr;
  a.va_c0 = e->ncell_tile + e->ncell_warp;
  a.va_c1 = a.va_c0 + e->ncell_va;
  a.n_ap = (int)ap.size();
  a.hist_len = (1 << e->radix_bits) * e->ntiles;
  if (e->nsys > 0) {
    SPC_CUDA(e, cudaMemcpyAsync(e->d_sys, table.data(), table.size() * sizeof(SysDesc),
                                cudaMemcpyHostToDevice, e->stream));
    if (!ap.empty())
      SPC_CUDA(e, cudaMemcpyAsync(e->d_ap, ap.data(), ap.size() * sizeof(int), cudaMemcpyHostToDevice,
                                  e->stream));
    if (!ap_all.empty())
      SPC_CUDA(e, cudaMemcpyAsync(e->d_ap_all, ap_all.data(), ap_all.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, e->stream));
    const int g = std::max(e->n_active, e->ncell_total);
    k_layout_maps<<<blocks_for(g, 256), 256, 0, e->stream>>>(e->d_sys, e->nsys, e->n_active, e->ncell_total,
                                                             (int *)a.sys_of_p, (int *)a.sys_of_c);
    SPC_LAUNCHED(e);
    // the histogram table must be zero before the next stage kernel
    SPC_CUDA(e, cudaMemsetAsync(e->hist, 0, (size_t)(1 << 11) * e->tile_cap * 4, e->stream));
    // host-side copies above read pageable memory: finish before `table` dies
    SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  }
  if (launch_shape(e) != shape0) drop_graph(e);
  e->dirty = false;
  return SPC_OK;
}

inline void mark(Engine *e, int slot) {
  if (e->profiling) cudaEventRecord(e->prof_ev[slot], e->stream);
}

inline int eval_cells(Engine *e, KArgs &a, int rk_form, int kq, double kcdt, bool marks = true);

// One evaluation's binning.  Verlet engines: refresh the Verlet-order copies
// of the stage state and rebuild the rows when the displacement test (or a
// stale build) asks for it; the rebuild is the cell-list binning plus the row
// build, all gated on the device flag.  verlet_ok = false (diagnostics, which
// need the reference's current cells) runs the cell-list binning and leaves
// the build stale.
inline int eval_stage(Engine *e, KArgs &a, int rk_form, int kq, double kcdt, bool verlet_ok = true) {
  // diagnostics visit each cell's members in ascending index: no sub-cells
  if (!verlet_ok) {
    a.cell_mid = nullptr;
    a.cell_near = nullptr;
  }
  if (!e->verlet) return eval_cells(e, a, rk_form, kq, kcdt);
  if (!verlet_ok) {
    e->verlet_stale = true;
    return eval_cells(e, a, rk_form, kq, kcdt);
  }
  const int n = e->n_active;
  cudaStream_t st = e->stream;
  // the gather and the rebuild see the build tables; the caller's arguments
  // (and the cell-list path's) leave them null
  KArgs b = a;
  b.gate = e->vflags;
  b.vsys = e->vsys;
  b.vcell = e->vcell;
  if (e->precision == SPC_PRECISION_FP32C)
    k_vgather<kPrecFP32C><<<blocks_for(n, 256), 256, 0, st>>>(b, rk_form, kq, kcdt);
  else
    k_vgather<kPrecFP64><<<blocks_for(n, 256), 256, 0, st>>>(b, rk_form, kq, kcdt);
  SPC_LAUNCHED(e);
  mark(e, 1);
  SPC_TRY(eval_cells(e, b, rk_form, kq, kcdt, false));
  mark(e, 2);
  k_verlet_build<<<std::min(std::max(e->ncell_total, 1), 152 * 16), kVThreads, 0, st>>>(b);
  SPC_LAUNCHED(e);
  mark(e, 3);
  a.skeys = b.skeys;
  a.svals = b.svals;
  return SPC_OK;
}

// Cell-list binning: stage, sort, cell bounds, cell-order gather.  marks:
// record the profiling events after each part.
inline int eval_cells(Engine *e, KArgs &a, int rk_form, int kq, double kcdt, bool marks) {
  const int n = e->n_active;
  cudaStream_t st = e->stream;
  const int bits = e->radix_bits;
  k_stage<<<blocks_for(n, kStageThreads), kStageThreads, 0, st>>>(a, rk_form, kq, kcdt, bits, e->hist);
  SPC_LAUNCHED(e);
  if (marks) mark(e, 1);
  uint32_t *kin = a.keys, *vin = a.vals, *kout = e->keys_alt, *vout = e->vals_alt;
  for (int pass = 0; pass < e->sort_passes; ++pass) {
    const int shift = pass * bits;
    if (pass > 0) k_radix_hist<<<e->ntiles, kSortThreads, 0, st>>>(kin, n, shift, bits, e->hist, a.gate);
    if (e->ntiles <= kScanGroup) {
      k_scan_digits<<<1, kScanThreads, 0, st>>>(e->hist, e->ntiles, bits, a.gate);
    } else {
      const int ng = (e->ntiles + kScanGroup - 1) / kScanGroup;
      const dim3 grid(ng, blocks_for(1 << bits, 256));
      k_scan_group_sums<<<grid, 256, 0, st>>>(e->hist, e->ntiles, bits, e->part, a.gate);
      k_scan_digits<<<1, kScanThreads, 0, st>>>(e->part, ng, bits, a.gate);
      k_scan_group_apply<<<grid, 256, 0, st>>>(e->hist, e->ntiles, bits, e->part, a.gate);
    }
    if (e->ntiles < kScatterSplitBelow)
      k_radix_scatter<4><<<e->ntiles * 4, kSortThreads, scatter_smem_bytes(bits), st>>>(
          kin, vin, kout, vout, n, shift, bits, e->hist, a.gate);
    else
      k_radix_scatter<1><<<e->ntiles, kSortThreads, scatter_smem_bytes(bits), st>>>(
          kin, vin, kout, vout, n, shift, bits, e->hist, a.gate);
    SPC_LAUNCHED(e);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (marks) mark(e, 2);
  a.skeys = kin;
  a.svals = vin;
  if (e->precision == SPC_PRECISION_FP32C)
    k_gather<kPrecFP32C><<<blocks_for(n + 1, 256), 256, 0, st>>>(a);
  else if (e->precision == SPC_PRECISION_FP32X)
    k_gather<kPrecFP32X><<<blocks_for(n + 1, 256), 256, 0, st>>>(a);
  else
    k_gather<kPrecFP64><<<blocks_for(n + 1, 256), 256, 0, st>>>(a);
  SPC_LAUNCHED(e);
  if (a.units && e->ncell_tile > 0 && !e->verlet) {  // the cell units of this evaluation
    if (e->precision == SPC_PRECISION_FP32C)
      k_list_units<kTileCap><<<blocks_for(e->ncell_tile, 128), 128, 0, st>>>(a);
    else
      k_list_units<kTileCapX><<<blocks_for(e->ncell_tile, 128), 128, 0, st>>>(a);
    SPC_LAUNCHED(e);
  }
  if (marks) mark(e, 3);
  return SPC_OK;
}

// The all-pairs kernel at 128 threads per CTA when its systems give at least
// two blocks per SM, else at one warp per CTA.
template <int PREC, int KIND>
void launch_allpairs(const KArgs &a, int epi, int items, int items_small, cudaStream_t st) {
  if (items >= 2 * 152)
    k_allpairs_pass<PREC, KIND, kAllPairsThreads><<<std::min(items, 152 * 16), kAllPairsThreads, 0, st>>>(a, epi);
  else
    k_allpairs_pass<PREC, KIND, kAllPairsThreadsSmall>
        <<<std::min(items_small, 152 * 32), kAllPairsThreadsSmall, 0, st>>>(a, epi);
}

template <int PREC, int KIND>
int launch_pass_t(Engine *e, const KArgs &a, int epi) {
  cudaStream_t st = e->stream;
  if constexpr (KIND == kKindNb) {
    // diagnostics count neighbours within rho for every model: the all-pairs
    // kernel takes every all-pairs system, the cell kernel every cell list
    KArgs b = a;
    b.ap_cells = e->d_ap_all;
    b.n_ap = e->n_ap_all;
    if (b.n_ap > 0) {
      launch_allpairs<PREC, KIND>(b, epi, e->ap_items_all, e->ap_items_all_small, st);
      SPC_LAUNCHED(e);
    }
    if (e->ncell_total > e->n_ap_all) {
      k_cell_pass<PREC, KIND><<<std::min(blocks_for(e->ncell_total, kPassWarps), 152 * 64), kPassThreads, 0,
                                st>>>(b, epi);
      SPC_LAUNCHED(e);
    }
    return SPC_OK;
  }
  if (a.n_ap > 0) {
    // FP32X all-pairs systems (rho > L/4: small boxes) run the FP64 pass
    constexpr int PA = PREC == kPrecFP32X ? kPrecFP64 : PREC;
    launch_allpairs<PA, KIND>(a, epi, e->ap_items, e->ap_items_small, st);
    SPC_LAUNCHED(e);
  }
  if constexpr (KIND != kKindNb && PREC != kPrecFP32X) {  // FP32X is refused with Verlet rows
    if (e->has_cells && e->verlet) {
      k_vtile<PREC, KIND><<<std::min(e->ncell_total, 152 * 256), kVThreads, 0, st>>>(a, epi);
      SPC_LAUNCHED(e);
      return SPC_OK;
    }
  }
  if constexpr (PREC == kPrecFP64 && KIND != kKindNb) {
    if (e->ncell_va > 0) {
      k_va_pass<KIND><<<std::min(e->ncell_va, 152 * 64), kVAThreads, 0, st>>>(a, epi);
      SPC_LAUNCHED(e);
    }
  }
  if (e->has_cells) {
    {
      if (e->ncell_tile > 0) {
        const int grid = std::min(e->ncell_tile * std::max(a.tile_split, 1), 152 * 256);
        if constexpr ((PREC == kPrecFP32C || PREC == kPrecFP32X) && KIND != kKindNb) {
          if (a.units) {
            // the cell units (listed after the gather) run beside the
            // cell-tile kernel, each filling the SMs the other leaves idle.
            // One CTA per unit up to 16 per SM (CTAs past the unit count
            // return at once, a larger count is taken in turn): measured
            // against 3, 4, 6, 7 and 10 per SM, the most units in flight won.
            SPC_CUDA(e, cudaEventRecord(e->fork_ev, st));
            SPC_CUDA(e, cudaStreamWaitEvent(e->side, e->fork_ev, 0));
            if constexpr (PREC == kPrecFP32C)
              k_units_fp32c<KIND><<<152 * 16, kTileThreads32, 0, e->side>>>(a, epi);
            else
              k_units_fp32x<KIND><<<152 * 16, kTileThreads32, 0, e->side>>>(a, epi);
            SPC_LAUNCHED(e);
            SPC_CUDA(e, cudaEventRecord(e->join_ev, e->side));
          }
        }
        if constexpr (PREC == kPrecFP32C) {
          if (a.units)
            k_tile_fp32c<KIND, true><<<grid, kTileThreads32, 0, st>>>(a, epi);
          else
            k_tile_fp32c<KIND, false><<<grid, kTileThreads32, 0, st>>>(a, epi);
        } else if constexpr (PREC == kPrecFP32X) {
          if (a.units)
            k_tile_fp32x<KIND, true><<<grid, kTileThreads32, 0, st>>>(a, epi);
          else
            k_tile_fp32x<KIND, false><<<grid, kTileThreads32, 0, st>>>(a, epi);
        } else
          k_tile_fp64<KIND><<<grid, kTileThreads64, 0, st>>>(a, epi);
        SPC_LAUNCHED(e);
        if constexpr ((PREC == kPrecFP32C || PREC == kPrecFP32X) && KIND != kKindNb)
          if (a.units) SPC_CUDA(e, cudaStreamWaitEvent(st, e->join_ev, 0));
      }
      if (e->ncell_warp > 0) {
        const int grid = std::min(blocks_for(e->ncell_warp, kWarpPassWarps), 152 * 64);
        if constexpr (PREC == kPrecFP32C)
          k_warp_fp32c<KIND><<<grid, kWarpPassThreads, 0, st>>>(a, epi);
        else if constexpr (PREC == kPrecFP32X)
          k_warp_fp32x<KIND><<<grid, kWarpPassThreads, 0, st>>>(a, epi);
        else
          k_warp_fp64<KIND><<<grid, kWarpPassThreads, 0, st>>>(a, epi);
        SPC_LAUNCHED(e);
      }
      if constexpr (PREC == kPrecFP32X && KIND != kKindNb) {
        // the neighbour kernels wrote the sums; the FP64 epilogues run densely
        if (e->ncell_tile + e->ncell_warp > 0) {
          k_epilogue_fp32x<KIND><<<blocks_for(e->n_active, 256), 256, 0, st>>>(a, epi);
          SPC_LAUNCHED(e);
        }
      }
    }
  }
  return SPC_OK;
}

inline int launch_pass(Engine *e, const KArgs &a, int kind, int epi) {
  if (kind == kKindNb) return launch_pass_t<kPrecFP64, kKindNb>(e, a, epi);
  const bool cos2 = kind == kKindCos2;
  switch (e->precision) {
    case SPC_PRECISION_FP32C:
      return cos2 ? launch_pass_t<kPrecFP32C, kKindCos2>(e, a, epi) : launch_pass_t<kPrecFP32C, kKindSin>(e, a, epi);
    case SPC_PRECISION_FP32X:
      return cos2 ? launch_pass_t<kPrecFP32X, kKindCos2>(e, a, epi) : launch_pass_t<kPrecFP32X, kKindSin>(e, a, epi);
    default:
      return cos2 ? launch_pass_t<kPrecFP64, kKindCos2>(e, a, epi) : launch_pass_t<kPrecFP64, kKindSin>(e, a, epi);
  }
}

// Enqueue one DoStep + wrap of every active system.  noise: pool-indexed
// device normals of this step, or null for Philox.
inline int enqueue_step(Engine *e, double dt, int step_off, const double *noise) {
  KArgs a = e->a;
  a.dt = dt;
  a.sdt = std::sqrt(dt);
  a.noise = noise;
  a.noise_m = noise_per_particle(e->stepper);
  a.step_off = step_off;
  switch (e->stepper) {
    case SPC_STEPPER_EULER:
      // EvaluateRhs(x, det, det, 0.0, dt) on the zero-filled det (StochasticEulerStepper.hpp:34-37)
      SPC_TRY(eval_stage(e, a, 1, -1, 0.0 * dt));
      SPC_TRY(launch_pass(e, a, kKindSin, kEpiEuler));
      mark(e, 4);
      break;
    case SPC_STEPPER_EULER_PTR:
      SPC_TRY(eval_stage(e, a, 0, -1, 0.0));
      SPC_TRY(launch_pass(e, a, kKindSin, kEpiEulerPtr));
      mark(e, 4);
      break;
    case SPC_STEPPER_SRK:
      SPC_TRY(eval_stage(e, a, 0, -1, 0.0));
      SPC_TRY(launch_pass(e, a, kKindSin, kEpiSrk1));
      mark(e, 4);
      SPC_TRY(launch_pass(e, a, kKindCos2, kEpiSrk2));
      break;
    case SPC_STEPPER_RK4: {
      // RungeKutta4Stepper.cpp:31-45: k_coef 0, 1/2, 1/2, 1 on k1, k1, k2, k3
      const double coef[4] = {0.0, 0.5, 0.5, 1.0};
      const int kprev[4] = {0, 0, 1, 2};
      for (int s = 0; s < 4; ++s) {
        if (s > 0) e->profiling = false;  // phases are timed on the first stage
        SPC_TRY(eval_stage(e, a, 1, kprev[s], coef[s] * dt));
        a.kq_out = s;
        SPC_TRY(launch_pass(e, a, kKindSin, s == 3 ? kEpiRk4Combine : kEpiRkK));
        if (s == 0) mark(e, 4);
      }
      break;
    }
    default:
      return fail(e, SPC_ERR_INVALID, "unknown stepper %d", e->stepper);
  }
  return SPC_OK;
}

// Host mirror of the per-call step bookkeeping (k_begin_call / k_end_call).
inline void mirror_call(Engine *e, int nsteps) {
  for (int slot : e->order) {
    SysHost &h = e->slots[slot];
    const long long b = std::max(0ll, std::min<long long>(nsteps, h.remaining));
    h.step += (unsigned long long)b;
    h.remaining -= b;
  }
}

// nsteps steps of every active system (eagerly launched or as a replayed
// CUDA graph).  noise (single-system injection) is consumed per step.
// The graph of nsteps steps at dt, captured and instantiated unless the
// cached one fits (the layout must be current).
inline int engine_capture(Engine *e, double dt, int nsteps) {
  if (e->graph && e->graph_steps == nsteps && e->graph_dt == dt) return SPC_OK;
  drop_graph(e);
  const int sb = blocks_for(e->nsys, 128);
  cudaGraph_t g = nullptr;
  SPC_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  int rc = SPC_OK;
  k_begin_call<<<sb, 128, 0, e->stream>>>(e->d_sys, e->nsys, nsteps);
  for (int s = 0; s < nsteps && rc == SPC_OK; ++s) rc = enqueue_step(e, dt, s, nullptr);
  k_end_call<<<sb, 128, 0, e->stream>>>(e->d_sys, e->nsys);
  cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
  if (rc != SPC_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ce != cudaSuccess) return fail(e, SPC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
  e->graph_nodes = 0;
  cudaGraphGetNodes(g, nullptr, &e->graph_nodes);
  ce = cudaGraphInstantiate(&e->graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) {
    e->graph = nullptr;
    return fail(e, SPC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
  }
  e->graph_steps = nsteps;
  e->graph_dt = dt;
  return SPC_OK;
}

// Captures (without launching) the step graph a later graph call of nsteps
// steps at dt will replay, so that its capture cost falls outside whatever
// the caller times.
inline int engine_prepare_graph(Engine *e, double dt, int nsteps) {
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  if (e->nsys == 0 || nsteps <= 0) return SPC_OK;
  return engine_capture(e, dt, nsteps);
}

inline int engine_steps(Engine *e, double dt, int nsteps, bool use_graph, const double *noise_base,
                        long long noise_per_step) {
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  if (e->nsys == 0 || nsteps == 0) return SPC_OK;
  SPC_TRY(verlet_prepare(e));
  const int sb = blocks_for(e->nsys, 128);
  if (!use_graph) {
    k_begin_call<<<sb, 128, 0, e->stream>>>(e->d_sys, e->nsys, nsteps);
    SPC_LAUNCHED(e);
    for (int s = 0; s < nsteps; ++s)
      SPC_TRY(enqueue_step(e, dt, s, noise_base ? noise_base + (long long)s * noise_per_step : nullptr));
    k_end_call<<<sb, 128, 0, e->stream>>>(e->d_sys, e->nsys);
    SPC_LAUNCHED(e);
  } else {
    SPC_TRY(engine_capture(e, dt, nsteps));
    SPC_CUDA(e, cudaGraphLaunch(e->graph, e->stream));
  }
  mirror_call(e, nsteps);
  return SPC_OK;
}

inline int engine_set_tuning(Engine *e, int key, double value) {
  if (key == SPC_TUNE_VERLET_ROW_LIMIT) {
    if (!e->verlet) return fail(e, SPC_ERR_STATE, "no Verlet rows on this handle");
    if (!(value >= 1.0) || !(value <= (double)e->vcap_alloc))
      return fail(e, SPC_ERR_INVALID, "row limit must be in [1, %d]", e->vcap_alloc);
    e->a.vcap = (int)value;
    e->verlet_stale = true;  // rebuild the rows under the new limit
    drop_graph(e);
    return SPC_OK;
  }
  if (key == SPC_TUNE_CELL_UNITS) {
    if (value != 0.0 && value != 1.0) return fail(e, SPC_ERR_INVALID, "cell units must be 0 or 1");
    if (value == 1.0 && e->precision == SPC_PRECISION_FP64)
      return fail(e, SPC_ERR_INVALID, "cell units apply to the FP32C and FP32X cell-tile passes");
    if ((int)value != e->cell_units_tune) {
      e->cell_units_tune = (int)value;
      e->dirty = true;
    }
    return SPC_OK;
  }
  if (key == SPC_TUNE_SUBCELLS) {
    if (value != 0.0 && value != 1.0) return fail(e, SPC_ERR_INVALID, "sub-cells must be 0 or 1");
    if (value == 1.0 && (e->precision == SPC_PRECISION_FP64 || e->verlet))
      return fail(e, SPC_ERR_INVALID, "sub-cells apply to the FP32C and FP32X cell-list passes");
    if ((int)value != e->subcells_tune) {
      e->subcells_tune = (int)value;
      e->dirty = true;
    }
    return SPC_OK;
  }
  if (key == SPC_TUNE_TILE_SPLIT) {
    if (!(value >= 0.0) || !(value <= 8.0) || value != std::floor(value))
      return fail(e, SPC_ERR_INVALID, "tile split must be an integer in [0, 8]");
    if ((int)value != e->tile_split_tune) {
      e->tile_split_tune = (int)value;
      e->dirty = true;
    }
    return SPC_OK;
  }
  if (key == SPC_TUNE_SPARSE_BELOW) {
    if (!(value >= 0.0) || !std::isfinite(value)) return fail(e, SPC_ERR_INVALID, "sparse_below must be >= 0");
    if (value != e->sparse_below) {
      e->sparse_below = value;
      e->dirty = true;  // the next step lays the systems out again
    }
    return SPC_OK;
  }
  return fail(e, SPC_ERR_INVALID, "unknown tuning key %d", key);
}

inline int engine_get_tuning(const Engine *e, int key, double *value) {
  if (key == SPC_TUNE_VERLET_ROW_LIMIT) {
    *value = e->verlet ? (double)e->a.vcap : 0.0;
    return SPC_OK;
  }
  if (key == SPC_TUNE_SPARSE_BELOW) {
    *value = e->sparse_below;
    return SPC_OK;
  }
  if (key == SPC_TUNE_CELL_UNITS) {
    *value = (double)e->cell_units_tune;
    return SPC_OK;
  }
  if (key == SPC_TUNE_SUBCELLS) {
    *value = (double)e->subcells_tune;
    return SPC_OK;
  }
  if (key == SPC_TUNE_TILE_SPLIT) {  // the split in effect
    *value = (double)tile_split_for(e->tile_split_tune);
    return SPC_OK;
  }
  return fail(nullptr, SPC_ERR_INVALID, "unknown tuning key %d", key);
}

// Kernel-choice candidates of the cell-list passes: the threshold below which
// systems take the warp-per-cell kernels (all cell-tile, the default, all
// warp-per-cell) and the cell-tile kernels' CTAs per cell.
struct TuneCand {
  double sparse;
  int split;
  int units;
  int subcells;
};

// The kernel-choice candidates; cell units (float forms) with one and two
// CTAs per cell, and sub-cells (float forms; their units replace the
// cell-tile kernel for all but the longest lists, so one CTA per cell).
inline std::vector<TuneCand> kernel_candidates(int precision) {
  std::vector<TuneCand> c;
  for (double sb : {0.0, kSparseBelowDefault, 1e9})
    for (int split : {1, 2, 4}) {
      if (sb == 1e9 && split != 1) continue;  // no cell-tile systems left: the split does nothing
      c.push_back({sb, split, 0, 0});
    }
  if (precision != SPC_PRECISION_FP64) {
    for (double sb : {0.0, kSparseBelowDefault})
      for (int split : {1, 2}) c.push_back({sb, split, 1, 0});
    for (double sb : {0.0, kSparseBelowDefault}) c.push_back({sb, 1, 1, 1});
  }
  return c;
}

// Times every kernel-choice candidate on the engine's current state and keeps
// the fastest.  Each candidate runs trial steps once to settle (layout, first
// launches) and once under CUDA events; after each run the pool state (and
// RK4's rates) and every system's step counters are put back, so the state the
// caller continues from is the one it had.  out[k] (k < cap) gets candidate k
// with its milliseconds per step.  Verlet engines keep their rows (the knobs
// apply to the cell list): their one candidate is the current setting.
inline int engine_retune(Engine *e, double dt, int trial, spc_tuning *out, int cap, int *count, int *best) {
  if (e->injecting) return fail(e, SPC_ERR_STATE, "retuning runs Philox-noise steps; clear injected noise first");
  if (trial <= 0) return fail(e, SPC_ERR_INVALID, "trial_steps must be positive");
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  std::vector<TuneCand> cands = e->verlet ? std::vector<TuneCand>{{e->sparse_below, e->tile_split_tune,
                                                                    e->cell_units_tune, e->subcells_tune}}
                                          : kernel_candidates(e->precision);
  const size_t P = (size_t)e->pool_cap;
  std::vector<double *> live = {e->a.x, e->a.y, e->a.phi};
  if (e->stepper == SPC_STEPPER_RK4)
    for (int q = 0; q < 4; ++q) live.insert(live.end(), {e->a.kx[q], e->a.ky[q], e->a.kphi[q]});
  double *save = nullptr;
  SPC_CUDA(e, cudaMalloc(&save, live.size() * P * sizeof(double)));
  std::vector<std::pair<unsigned long long, long long>> ctr;
  for (int s : e->order) ctr.push_back({e->slots[s].step, e->slots[s].remaining});
  auto copy_all = [&](bool to_save) -> cudaError_t {
    for (size_t k = 0; k < live.size(); ++k) {
      double *dst = to_save ? save + k * P : live[k];
      const double *src = to_save ? live[k] : save + k * P;
      const cudaError_t ce = cudaMemcpyAsync(dst, src, P * sizeof(double), cudaMemcpyDeviceToDevice, e->stream);
      if (ce != cudaSuccess) return ce;
    }
    return cudaSuccess;
  };
  auto restore = [&]() -> int {
    const cudaError_t ce = copy_all(false);
    if (ce != cudaSuccess) return fail(e, SPC_ERR_CUDA, "retune restore: %s", cudaGetErrorString(ce));
    size_t i = 0;
    for (int s : e->order) {
      e->slots[s].step = ctr[i].first;
      e->slots[s].remaining = ctr[i].second;
      ++i;
    }
    e->dirty = true;  // the device table is rebuilt from the restored counters
    return SPC_OK;
  };
  const double sb0 = e->sparse_below;
  const int split0 = e->tile_split_tune, units0 = e->cell_units_tune, sub0 = e->subcells_tune;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaError_t ce = copy_all(true);
  if (ce == cudaSuccess) ce = cudaEventCreate(&ev[0]);
  if (ce == cudaSuccess) ce = cudaEventCreate(&ev[1]);
  int rc = ce == cudaSuccess ? SPC_OK : fail(e, SPC_ERR_CUDA, "retune: %s", cudaGetErrorString(ce));
  int best_k = 0;
  double best_ms = 1e300;
  for (size_t k = 0; k < cands.size() && rc == SPC_OK; ++k) {
    e->sparse_below = cands[k].sparse;
    e->tile_split_tune = cands[k].split;
    e->cell_units_tune = cands[k].units;
    e->subcells_tune = cands[k].subcells;
    e->dirty = true;
    rc = engine_steps(e, dt, trial, false, nullptr, 0);
    if (rc == SPC_OK) rc = restore();
    if (rc == SPC_OK) rc = engine_layout(e);  // outside the timed region
    if (rc == SPC_OK && cudaEventRecord(ev[0], e->stream) != cudaSuccess) rc = fail(e, SPC_ERR_CUDA, "event");
    if (rc == SPC_OK) rc = engine_steps(e, dt, trial, false, nullptr, 0);
    float ms = 0.0f;
    if (rc == SPC_OK && (cudaEventRecord(ev[1], e->stream) != cudaSuccess ||
                         cudaEventSynchronize(ev[1]) != cudaSuccess ||
                         cudaEventElapsedTime(&ms, ev[0], ev[1]) != cudaSuccess))
      rc = fail(e, SPC_ERR_CUDA, "retune timing");
    if (rc == SPC_OK) rc = restore();
    const double per = (double)ms / trial;
    if (rc == SPC_OK && (int)k < cap && out) {
      out[k].neighbour = e->verlet ? SPC_NEIGHBOUR_VERLET : SPC_NEIGHBOUR_CELL;
      out[k].tile_split = tile_split_for(cands[k].split);
      out[k].skin = 0.0;
      out[k].sparse_below = cands[k].sparse;
      out[k].ms_per_step = per;
      out[k].cell_units = cands[k].units;
      out[k].subcells = cands[k].subcells;
    }
    if (rc == SPC_OK && per < best_ms) {
      best_ms = per;
      best_k = (int)k;
    }
  }
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  cudaStreamSynchronize(e->stream);
  cudaFree(save);
  if (rc != SPC_OK) {  // keep the caller's settings
    e->sparse_below = sb0;
    e->tile_split_tune = split0;
    e->cell_units_tune = units0;
    e->subcells_tune = sub0;
    e->dirty = true;
    return rc;
  }
  e->sparse_below = cands[best_k].sparse;
  e->tile_split_tune = cands[best_k].split;
  e->cell_units_tune = cands[best_k].units;
  e->subcells_tune = cands[best_k].subcells;
  e->dirty = true;
  if (count) *count = (int)cands.size();
  if (best) *best = best_k;
  return SPC_OK;
}

// nsteps eagerly launched steps with CUDA events between the phases; out_ms[k]
// is the mean per step of: stage, sort, gather, first pass, rest of the step,
// whole step.
inline int engine_profile(Engine *e, double dt, int nsteps, double *out_ms) {
  if (e->injecting) return fail(e, SPC_ERR_STATE, "profiling uses Philox noise");
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  SPC_TRY(verlet_prepare(e));
  for (int k = 0; k < 6; ++k) {
    out_ms[k] = 0.0;
    if (!e->prof_ev[k]) SPC_CUDA(e, cudaEventCreate(&e->prof_ev[k]));
  }
  if (e->nsys == 0 || nsteps <= 0) return SPC_OK;
  const int sb = blocks_for(e->nsys, 128);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  k_begin_call<<<sb, 128, 0, e->stream>>>(e->d_sys, e->nsys, nsteps);
  SPC_LAUNCHED(e);
  for (int s = 0; s < nsteps; ++s) {
    // phase marks: 0 start, 1 after stage, 2 after sort, 3 after gather,
    // 4 after the first pass, 5 end of step
    SPC_CUDA(e, cudaEventRecord(e->prof_ev[0], e->stream));
    e->profiling = true;
    const int rc = enqueue_step(e, dt, s, nullptr);
    e->profiling = false;
    if (rc != SPC_OK) return rc;
    SPC_CUDA(e, cudaEventRecord(e->prof_ev[5], e->stream));
    SPC_CUDA(e, cudaEventSynchronize(e->prof_ev[5]));
    float ms[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 1; k <= 5; ++k) SPC_CUDA(e, cudaEventElapsedTime(&ms[k], e->prof_ev[k - 1], e->prof_ev[k]));
    for (int k = 0; k < 5; ++k) acc[k] += ms[k + 1];
    float tot = 0.0f;
    SPC_CUDA(e, cudaEventElapsedTime(&tot, e->prof_ev[0], e->prof_ev[5]));
    acc[5] += tot;
  }
  k_end_call<<<sb, 128, 0, e->stream>>>(e->d_sys, e->nsys);
  SPC_LAUNCHED(e);
  mirror_call(e, nsteps);
  for (int k = 0; k < 6; ++k) out_ms[k] = acc[k] / nsteps;
  return SPC_OK;
}

// Per-system overwrite of the device table's step counter (the layout copy
// is rebuilt from the host mirror, so this only marks the layout dirty).
inline void engine_set_step(Engine *e, int slot, unsigned long long step) {
  e->slots[slot].step = step;
  e->dirty = true;
}

// AoS <-> pool range of one system
inline int engine_upload(Engine *e, int slot, const double *aos3n) {
  const SysHost &h = e->slots[slot];
  SPC_CUDA(e, cudaMemcpyAsync(e->aos, aos3n, 3 * (size_t)h.n * 8, cudaMemcpyHostToDevice, e->stream));
  k_aos_to_soa<<<blocks_for(h.n, 256), 256, 0, e->stream>>>(e->aos, h.n, e->a.x + h.pool_p0,
                                                            e->a.y + h.pool_p0, e->a.phi + h.pool_p0);
  SPC_LAUNCHED(e);
  return SPC_OK;
}

inline int engine_download(Engine *e, int slot, double *aos3n) {
  const SysHost &h = e->slots[slot];
  k_soa_to_aos<<<blocks_for(h.n, 256), 256, 0, e->stream>>>(e->a.x + h.pool_p0, e->a.y + h.pool_p0,
                                                            e->a.phi + h.pool_p0, h.n, e->aos);
  SPC_LAUNCHED(e);
  SPC_CUDA(e, cudaMemcpyAsync(aos3n, e->aos, 3 * (size_t)h.n * 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  return SPC_OK;
}

inline int engine_upload_omega(Engine *e, int slot, const double *omega) {
  SysHost &h = e->slots[slot];
  SPC_CUDA(e, cudaMemcpyAsync((double *)e->a.omega + h.pool_p0, omega, (size_t)h.n * 8,
                              cudaMemcpyHostToDevice, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  h.omega_set = true;
  return SPC_OK;
}

inline int engine_order_global(Engine *e, int slot, double *R, double *psi) {
  const SysHost &h = e->slots[slot];
  const int blocks = std::min(blocks_for(h.n, 256), e->order_blocks);
  k_order_sum<<<blocks, 256, 0, e->stream>>>(e->a.phi + h.pool_p0, h.n, e->order_part);
  SPC_LAUNCHED(e);
  std::vector<double> part(2 * (size_t)blocks);
  SPC_CUDA(e, cudaMemcpyAsync(part.data(), e->order_part, part.size() * 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  double re = 0.0, im = 0.0;
  for (int b = 0; b < blocks; ++b) {
    re += part[2 * b];
    im += part[2 * b + 1];
  }
  re /= (double)h.n;
  im /= (double)h.n;
  if (R) *R = std::hypot(re, im);
  if (psi) *psi = std::atan2(im, re);
  return SPC_OK;
}

// Global and local order parameters of every system at once: one local-order
// pass over the whole layout (pool-indexed results), the pool phases and
// those results copied to the host, and FP64 sums per system there.  Entries
// [0, cap) are written; slots without a system get NaN.
inline int engine_order_all(Engine *e, int cap, double *R, double *psi, double *R_local) {
  SPC_TRY(engine_layout(e));
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (int s = 0; s < cap; ++s) {
    if (R) R[s] = nan;
    if (psi) psi[s] = nan;
    if (R_local) R_local[s] = nan;
  }
  if (e->nsys == 0) return SPC_OK;
  const size_t P = (size_t)e->pool_cap;
  std::vector<double> phi(P), r;
  if (R_local) {
    KArgs a = e->a;
    a.out_r = e->aos;
    SPC_TRY(eval_stage(e, a, 0, -1, 0.0, false));
    SPC_TRY(launch_pass(e, a, kKindNb, kEpiLocalOrder));
    r.resize(P);
    SPC_CUDA(e, cudaMemcpyAsync(r.data(), a.out_r, P * 8, cudaMemcpyDeviceToHost, e->stream));
  }
  SPC_CUDA(e, cudaMemcpyAsync(phi.data(), e->a.phi, P * 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  for (int s : e->order) {
    if (s >= cap) continue;
    const SysHost &h = e->slots[s];
    double re = 0.0, im = 0.0, rl = 0.0;
    for (int i = 0; i < h.n; ++i) {
      re += std::cos(phi[h.pool_p0 + i]);
      im += std::sin(phi[h.pool_p0 + i]);
      if (R_local) rl += r[h.pool_p0 + i];
    }
    re /= (double)h.n;
    im /= (double)h.n;
    if (R) R[s] = std::hypot(re, im);
    if (psi) psi[s] = std::atan2(im, re);
    if (R_local) R_local[s] = rl / (double)h.n;
  }
  return SPC_OK;
}

}  // namespace spc
