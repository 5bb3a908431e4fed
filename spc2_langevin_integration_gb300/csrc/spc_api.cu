// C-ABI implementation (include/spc_gb300.h): one handle = one particle
// system resident in HBM as structure-of-arrays, one CUDA stream, and the
// kernel sequence of each stepper.  No CPU fallback: every entry point that
// computes launches the kernels in spc_kernels.cuh / spc_sort.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/spc_gb300.h"
#include "spc_kernels.cuh"
#include "spc_sort.cuh"
#include "spc_tile.cuh"

using namespace spc;

namespace {

std::mutex g_err_mu;
std::string g_last_error;

}  // namespace

struct spc_handle {
  spc_params p{};
  cudaEvent_t prof_ev[8] = {};  // phase boundaries while profiling (null otherwise)
  bool profiling = false;
  int n = 0;
  int device = 0;
  SysConst sc{};
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  KArgs a{};
  // sort scratch
  uint32_t *keys_alt = nullptr, *vals_alt = nullptr, *hist = nullptr;
  int ntiles = 0, sort_passes = 0, radix_bits = 8;
  const uint32_t *sorted_keys = nullptr, *sorted_vals = nullptr;
  double *aos = nullptr;       // AoS staging, 3N (4 x 3N for RK4 buffers)
  double *order_part = nullptr;
  int order_blocks = 0;
  unsigned long long *d_step = nullptr, *d_clamped = nullptr;
  uint64_t step = 0;
  bool uploaded = false, omega_set = false, scratch_k = false;
  // injected noise
  double *d_noise = nullptr;
  int64_t noise_count = 0, noise_cursor = 0;
  bool injecting = false;
  // CUDA graph cache
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  double graph_dt = 0.0;
  std::string err;
};

namespace {

int fail(spc_handle *h, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = buf;
  return code;
}

#define SPC_CUDA(h, call)                                                                    \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail((h), e_ == cudaErrorMemoryAllocation ? SPC_ERR_NOMEM : SPC_ERR_CUDA,       \
                  "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
  } while (0)

#define SPC_LAUNCHED(h) SPC_CUDA(h, cudaGetLastError())

template <class T>
int dalloc(spc_handle *h, T **ptr, size_t count) {
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess)
    return fail(h, SPC_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T),
                cudaGetErrorString(e));
  h->allocs.push_back(p);
  *ptr = (T *)p;
  return SPC_OK;
}

// A positive finite power of two (then x / L equals x * (1 / L) exactly).
inline int is_pow2(double L) {
  int e = 0;
  return std::frexp(L, &e) == 0.5 ? 1 : 0;
}

inline int blocks_for(long long n, int threads) { return (int)((n + threads - 1) / threads); }

int noise_m(const spc_params &p) {
  switch (p.stepper) {
    case SPC_STEPPER_SRK: return 2;
    case SPC_STEPPER_RK4: return 0;
    default: return 1;
  }
}

// The 11-bit scatter needs more than the default 48 KB of dynamic shared
// memory; the attribute is set with the device current (not a stream
// operation, so never inside a capture).
cudaError_t set_kernel_attributes() {
  return cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)scatter_smem_bytes(11));
}

int set_device(spc_handle *h) {
  SPC_CUDA(h, cudaSetDevice(h->device));
  return SPC_OK;
}

// ---------------------------------------------------------------------------
// One evaluation's binning: stage, sort, cell bounds, cell-order gather.
void mark(spc_handle *h, int slot) {
  if (h->profiling) cudaEventRecord(h->prof_ev[slot], h->stream);
}

int eval_stage(spc_handle *h, KArgs &a, int rk_form, int kq, double kcdt) {
  const int n = h->n;
  cudaStream_t st = h->stream;
  const int bits = h->radix_bits;
  k_stage<<<blocks_for(n, kStageThreads), kStageThreads, 0, st>>>(a, rk_form, kq, kcdt,
                                                                   h->sc.allpairs ? 0 : bits, h->hist);
  SPC_LAUNCHED(h);
  mark(h, 1);
  if (h->sc.allpairs) {
    if (h->p.precision == SPC_PRECISION_FP32C) {
      k_fill_cs<<<blocks_for(n, 256), 256, 0, st>>>(a);
      SPC_LAUNCHED(h);
    }
    mark(h, 2);
    mark(h, 3);
    return SPC_OK;
  }
  uint32_t *kin = a.keys, *vin = a.vals, *kout = h->keys_alt, *vout = h->vals_alt;
  for (int pass = 0; pass < h->sort_passes; ++pass) {
    const int shift = pass * bits;
    if (pass > 0) k_radix_hist<<<h->ntiles, kSortThreads, 0, st>>>(kin, n, shift, bits, h->hist);
    k_scan_digits<<<1, kScanThreads, 0, st>>>(h->hist, h->ntiles, bits);
    k_radix_scatter<<<h->ntiles, kSortThreads, scatter_smem_bytes(bits), st>>>(kin, vin, kout, vout, n,
                                                                               shift, bits, h->hist);
    SPC_LAUNCHED(h);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  mark(h, 2);
  a.skeys = kin;
  a.svals = vin;
  if (h->p.precision == SPC_PRECISION_FP32C)
    k_gather<kPrecFP32C><<<blocks_for(n + 1, 256), 256, 0, st>>>(a);
  else
    k_gather<kPrecFP64><<<blocks_for(n + 1, 256), 256, 0, st>>>(a);
  SPC_LAUNCHED(h);
  mark(h, 3);
  return SPC_OK;
}

template <int PREC, int KIND>
int launch_pass_t(spc_handle *h, const KArgs &a, int epi) {
  cudaStream_t st = h->stream;
  if (h->sc.allpairs) {
    k_allpairs_pass<PREC, KIND><<<blocks_for(h->n, kAllPairsThreads), kAllPairsThreads, 0, st>>>(a, epi);
  } else if constexpr (KIND == kKindNb) {
    const int blocks = std::min(blocks_for(h->sc.ncell, kPassWarps), 152 * 64);
    k_cell_pass<PREC, KIND><<<blocks, kPassThreads, 0, st>>>(a, epi);
  } else if constexpr (PREC == kPrecFP32C) {
    k_tile_fp32c<KIND><<<std::min(h->sc.ncell, 152 * 256), kTileThreads32, 0, st>>>(a, epi);
  } else {
    k_tile_fp64<KIND><<<std::min(h->sc.ncell, 152 * 256), kTileThreads64, 0, st>>>(a, epi);
  }
  SPC_LAUNCHED(h);
  return SPC_OK;
}

int launch_pass(spc_handle *h, const KArgs &a, int kind, int epi, bool force_fp64 = false) {
  const bool fp32 = h->p.precision == SPC_PRECISION_FP32C && !force_fp64;
  if (kind == kKindSin)
    return fp32 ? launch_pass_t<kPrecFP32C, kKindSin>(h, a, epi) : launch_pass_t<kPrecFP64, kKindSin>(h, a, epi);
  if (kind == kKindCos2)
    return fp32 ? launch_pass_t<kPrecFP32C, kKindCos2>(h, a, epi) : launch_pass_t<kPrecFP64, kKindCos2>(h, a, epi);
  return launch_pass_t<kPrecFP64, kKindNb>(h, a, epi);
}

#define SPC_TRY(expr)          \
  do {                         \
    int rc_ = (expr);          \
    if (rc_ != SPC_OK) return rc_; \
  } while (0)

// Enqueue one DoStep + wrap.  noise: device normals of this step or null.
int enqueue_step(spc_handle *h, double dt, int step_off, const double *noise) {
  KArgs a = h->a;
  a.dt = dt;
  a.noise = noise;
  a.step_off = step_off;
  switch (h->p.stepper) {
    case SPC_STEPPER_EULER:
      // EvaluateRhs(x, det, det, 0.0, dt) on the zero-filled det (StochasticEulerStepper.hpp:34-37)
      SPC_TRY(eval_stage(h, a, 1, -1, 0.0 * dt));
      SPC_TRY(launch_pass(h, a, kKindSin, kEpiEuler));
      mark(h, 4);
      break;
    case SPC_STEPPER_EULER_PTR:
      SPC_TRY(eval_stage(h, a, 0, -1, 0.0));
      SPC_TRY(launch_pass(h, a, kKindSin, kEpiEulerPtr));
      mark(h, 4);
      break;
    case SPC_STEPPER_SRK:
      SPC_TRY(eval_stage(h, a, 0, -1, 0.0));
      SPC_TRY(launch_pass(h, a, kKindSin, kEpiSrk1));
      mark(h, 4);
      SPC_TRY(launch_pass(h, a, kKindCos2, kEpiSrk2));
      break;
    case SPC_STEPPER_RK4: {
      // RungeKutta4Stepper.cpp:31-45: k_coef 0, 1/2, 1/2, 1 on k1, k1, k2, k3
      const double coef[4] = {0.0, 0.5, 0.5, 1.0};
      const int kprev[4] = {0, 0, 1, 2};
      for (int s = 0; s < 4; ++s) {
        if (s > 0) h->profiling = false;  // phases are timed on the first stage
        SPC_TRY(eval_stage(h, a, 1, kprev[s], coef[s] * dt));
        a.kq_out = s;
        SPC_TRY(launch_pass(h, a, kKindSin, s == 3 ? kEpiRk4Combine : kEpiRkK));
        if (s == 0) mark(h, 4);
      }
      break;
    }
    default:
      return fail(h, SPC_ERR_INVALID, "unknown stepper %d", h->p.stepper);
  }
  return SPC_OK;
}

__global__ void k_set_u64(unsigned long long *p, unsigned long long v) { *p = v; }

// The device step counter is set by a kernel launch, which carries the value
// in its parameters: no host buffer has to outlive the call.
int write_step(spc_handle *h) {
  k_set_u64<<<1, 1, 0, h->stream>>>(h->d_step, (unsigned long long)h->step);
  SPC_LAUNCHED(h);
  return SPC_OK;
}

int validate(const spc_params *p, int n, spc_handle *h) {
  if (!p) return fail(h, SPC_ERR_INVALID, "params is NULL");
  if (n <= 0) return fail(h, SPC_ERR_INVALID, "n must be positive (got %d)", n);
  if (!(p->L > 0.0) || !std::isfinite(p->L)) return fail(h, SPC_ERR_INVALID, "L must be positive");
  if (!(p->rho > 0.0) || !std::isfinite(p->rho)) return fail(h, SPC_ERR_INVALID, "rho must be positive");
  if (!(p->D_phi >= 0.0)) return fail(h, SPC_ERR_INVALID, "D_phi must be >= 0");
  if (!std::isfinite(p->v0) || !std::isfinite(p->sigma) || !std::isfinite(p->alpha))
    return fail(h, SPC_ERR_INVALID, "v0, sigma, alpha must be finite");
  if (p->model != SPC_MODEL_CHIMERA && p->model != SPC_MODEL_VORTEX)
    return fail(h, SPC_ERR_INVALID, "unknown model %d", p->model);
  if (p->stepper < SPC_STEPPER_EULER || p->stepper > SPC_STEPPER_EULER_PTR)
    return fail(h, SPC_ERR_INVALID, "unknown stepper %d", p->stepper);
  if (p->model == SPC_MODEL_VORTEX && p->stepper != SPC_STEPPER_SRK)
    return fail(h, SPC_ERR_INVALID,
                "the vortex model's natural frequencies enter the stochastic Runge-Kutta update only");
  if (p->neighbour != SPC_NEIGHBOUR_CELL && p->neighbour != SPC_NEIGHBOUR_VERLET)
    return fail(h, SPC_ERR_INVALID, "unknown neighbour search %d", p->neighbour);
  if (p->precision != SPC_PRECISION_FP64 && p->precision != SPC_PRECISION_FP32C)
    return fail(h, SPC_ERR_INVALID, "unknown precision %d", p->precision);
  if (p->neighbour == SPC_NEIGHBOUR_VERLET && !(p->skin > 0.0))
    return fail(h, SPC_ERR_INVALID, "Verlet skin must be positive");
  if (p->rho <= 0.25 * p->L) {
    const double ncd = std::floor(p->L / p->rho);
    if (ncd > 46340.0) return fail(h, SPC_ERR_INVALID, "too many cells (L/rho = %g)", ncd);
  }
  return SPC_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

int spc_abi_version(void) { return SPC_ABI_VERSION; }

const char *spc_last_error(const spc_handle *h) {
  if (h) return h->err.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_last_error.c_str();
}

int spc_destroy(spc_handle *h) {
  if (!h) return SPC_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (cudaEvent_t e : h->prof_ev)
    if (e) cudaEventDestroy(e);
  for (void *p : h->allocs) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return SPC_OK;
}

int spc_create(const spc_params *p, int32_t n, spc_handle **out) {
  if (!out) return fail(nullptr, SPC_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate(p, n, nullptr);
  if (rc) return rc;
  spc_handle *h = new spc_handle();
  h->p = *p;
  h->n = n;
  auto bail = [&](int code) {
    std::string msg = h->err;
    spc_destroy(h);
    fail(nullptr, code, "%s", msg.c_str());
    return code;
  };
  if (cudaGetDevice(&h->device) != cudaSuccess) {
    h->err = "no CUDA device";
    return bail(SPC_ERR_CUDA);
  }
  if (set_kernel_attributes() != cudaSuccess) {
    h->err = "cudaFuncSetAttribute failed";
    return bail(SPC_ERR_CUDA);
  }
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    h->err = "cudaStreamCreate failed";
    return bail(SPC_ERR_CUDA);
  }
  SysConst &sc = h->sc;
  sc.n = n;
  sc.L = p->L;
  sc.rL = 1.0 / p->L;
  sc.rho2 = p->rho * p->rho;
  sc.v0 = p->v0;
  sc.sigma = p->sigma;
  sc.alpha = p->alpha;
  sc.D = p->D_phi;
  sc.allpairs = !(p->rho <= 0.25 * p->L);
  sc.nc = sc.allpairs ? 1 : std::max(1, (int)(p->L / p->rho));
  sc.ncell = sc.nc * sc.nc;
  sc.cell = p->L / sc.nc;
  sc.cell_f = (float)sc.cell;
  // prefilter band: a relative 3e-5 of rho^2 on each side, far wider than the
  // float error of the cell-relative dr^2 (about 3e-6 rho^2 for cells <= 4/3 rho)
  sc.lo2 = (float)(sc.rho2 * (1.0 - 3e-5));
  sc.hi2 = (float)(sc.rho2 * (1.0 + 3e-5));
  sc.exact_all = (p->flags & SPC_FLAG_EXACT_ALL) ? 1 : 0;
  sc.L_pow2 = is_pow2(p->L);

  KArgs &a = h->a;
  a.sc = sc;
  const size_t N = (size_t)n;
#define ALLOC(ptr, cnt)                         \
  do {                                          \
    if (dalloc(h, &(ptr), (cnt))) return bail(SPC_ERR_NOMEM); \
  } while (0)
  ALLOC(a.x, N);
  ALLOC(a.y, N);
  ALLOC(a.phi, N);
  double *omega = nullptr;
  ALLOC(omega, N);
  a.omega = omega;
  for (int q = 0; q < 4; ++q) {
    ALLOC(a.kx[q], N);
    ALLOC(a.ky[q], N);
    ALLOC(a.kphi[q], N);
  }
  ALLOC(a.st_x, N);
  ALLOC(a.st_y, N);
  ALLOC(a.st_phi, N);
  ALLOC(a.keys, N);
  ALLOC(a.vals, N);
  ALLOC(h->keys_alt, N);
  ALLOC(h->vals_alt, N);
  h->ntiles = (int)((N + kSortTile - 1) / kSortTile);
  int bits = 1;
  while (bits < 31 && (1u << bits) < (unsigned)sc.ncell) ++bits;
  // one pass of exactly the key width when it is at most 11 bits, else 8-bit passes
  h->radix_bits = (bits <= 11) ? bits : 8;
  h->sort_passes = (bits + h->radix_bits - 1) / h->radix_bits;
  ALLOC(h->hist, (size_t)(1 << h->radix_bits) * h->ntiles);
  ALLOC(a.cell_start, (size_t)sc.ncell + 1);
  ALLOC(a.sx, N);
  ALLOC(a.sy, N);
  ALLOC(a.sphi, N);
  ALLOC(a.fxy, N);
  ALLOC(a.cs, N);
  ALLOC(a.pidx, N);
  ALLOC(a.dphi_s, N);
  ALLOC(a.dphi_f, N);
  ALLOC(a.cnt_s, N);
  if (p->precision == SPC_PRECISION_FP32C && !sc.allpairs) ALLOC(a.nbmask, (size_t)kMaskWords * N);
  ALLOC(h->aos, 12 * N);
  h->order_blocks = std::min(blocks_for(n, 256), 1024);
  ALLOC(h->order_part, 2 * (size_t)h->order_blocks);
  ALLOC(h->d_step, 1);
  ALLOC(h->d_clamped, 1);
#undef ALLOC
  a.clamped = h->d_clamped;
  a.hist = h->hist;
  a.hist_len = (1 << h->radix_bits) * h->ntiles;
  a.step_base = h->d_step;
  a.seed = p->seed;
  a.system_id = p->system_id;
  a.is_vortex = p->model == SPC_MODEL_VORTEX;
  a.noise_m = noise_m(*p);
  // zero what the reference zero-initialises (k buffers, omega) and the counters
  cudaStream_t st = h->stream;
  if (cudaMemsetAsync(omega, 0, N * 8, st) != cudaSuccess) return bail(SPC_ERR_CUDA);
  for (int q = 0; q < 4; ++q) {
    if (cudaMemsetAsync(a.kx[q], 0, N * 8, st) || cudaMemsetAsync(a.ky[q], 0, N * 8, st) ||
        cudaMemsetAsync(a.kphi[q], 0, N * 8, st))
      return bail(SPC_ERR_CUDA);
  }
  if (cudaMemsetAsync(h->hist, 0, (size_t)a.hist_len * 4, st) ||
      cudaMemsetAsync(h->d_step, 0, 8, st) || cudaMemsetAsync(h->d_clamped, 0, 8, st) ||
      cudaMemsetAsync(a.x, 0, N * 8, st) || cudaMemsetAsync(a.y, 0, N * 8, st) ||
      cudaMemsetAsync(a.phi, 0, N * 8, st))
    return bail(SPC_ERR_CUDA);
  if (cudaStreamSynchronize(st) != cudaSuccess) return bail(SPC_ERR_CUDA);
  *out = h;
  return SPC_OK;
}

int spc_get_params(const spc_handle *h, spc_params *out, int32_t *n) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "handle is NULL");
  if (out) *out = h->p;
  if (n) *n = h->n;
  return SPC_OK;
}

int spc_upload_state(spc_handle *h, const double *aos3n) {
  if (!h || !aos3n) return fail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(set_device(h));
  const size_t N = h->n;
  SPC_CUDA(h, cudaMemcpyAsync(h->aos, aos3n, 3 * N * 8, cudaMemcpyHostToDevice, h->stream));
  k_aos_to_soa<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->aos, h->n, h->a.x, h->a.y, h->a.phi);
  SPC_LAUNCHED(h);
  h->uploaded = true;
  return SPC_OK;
}

int spc_download_state(spc_handle *h, double *aos3n) {
  if (!h || !aos3n) return fail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(set_device(h));
  const size_t N = h->n;
  k_soa_to_aos<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->a.x, h->a.y, h->a.phi, h->n, h->aos);
  SPC_LAUNCHED(h);
  SPC_CUDA(h, cudaMemcpyAsync(aos3n, h->aos, 3 * N * 8, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPC_OK;
}

int spc_upload_omega(spc_handle *h, const double *omega) {
  if (!h || !omega) return fail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(set_device(h));
  SPC_CUDA(h, cudaMemcpyAsync((void *)h->a.omega, omega, (size_t)h->n * 8, cudaMemcpyHostToDevice,
                              h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  h->omega_set = true;
  return SPC_OK;
}

int spc_download_rk4_buffers(spc_handle *h, double *out12n) {
  if (!h || !out12n) return fail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(set_device(h));
  const size_t N = h->n;
  for (int q = 0; q < 4; ++q) {
    k_soa_to_aos<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->a.kx[q], h->a.ky[q], h->a.kphi[q],
                                                                h->n, h->aos + q * 3 * N);
    SPC_LAUNCHED(h);
  }
  SPC_CUDA(h, cudaMemcpyAsync(out12n, h->aos, 12 * N * 8, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPC_OK;
}

int spc_upload_rk4_buffers(spc_handle *h, const double *in12n) {
  if (!h || !in12n) return fail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(set_device(h));
  const size_t N = h->n;
  SPC_CUDA(h, cudaMemcpyAsync(h->aos, in12n, 12 * N * 8, cudaMemcpyHostToDevice, h->stream));
  for (int q = 0; q < 4; ++q) {
    k_aos_to_soa<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->aos + q * 3 * N, h->n, h->a.kx[q],
                                                                h->a.ky[q], h->a.kphi[q]);
    SPC_LAUNCHED(h);
  }
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPC_OK;
}

int spc_noise_per_particle(const spc_handle *h) { return h ? noise_m(h->p) : 0; }

int spc_step(spc_handle *h, double *t_inout, double dt, int32_t nsteps) {
  if (!h || !t_inout) return fail(h, SPC_ERR_INVALID, "NULL argument");
  if (nsteps < 0) return fail(h, SPC_ERR_INVALID, "nsteps must be >= 0");
  if (!h->uploaded) return fail(h, SPC_ERR_STATE, "state not uploaded");
  if (h->p.model == SPC_MODEL_VORTEX && !h->omega_set)
    return fail(h, SPC_ERR_STATE, "vortex model: natural frequencies not uploaded");
  SPC_TRY(set_device(h));
  const int m = noise_m(h->p);
  const int64_t per_step = (int64_t)m * h->n;
  if (h->injecting && h->noise_cursor + per_step * nsteps > h->noise_count)
    return fail(h, SPC_ERR_NOISE, "injected noise: %lld normals left, %lld needed",
                (long long)(h->noise_count - h->noise_cursor), (long long)(per_step * nsteps));
  SPC_TRY(write_step(h));
  double t = *t_inout;
  for (int s = 0; s < nsteps; ++s) {
    t += dt;  // SimulationEngine.cpp:151
    const double *noise = nullptr;
    if (h->injecting && m > 0) {
      noise = h->d_noise + h->noise_cursor;
      h->noise_cursor += per_step;
    }
    SPC_TRY(enqueue_step(h, dt, s, noise));
  }
  h->step += (uint64_t)nsteps;
  *t_inout = t;
  return SPC_OK;
}

int spc_step_graph(spc_handle *h, double *t_inout, double dt, int32_t nsteps) {
  if (!h || !t_inout) return fail(h, SPC_ERR_INVALID, "NULL argument");
  if (nsteps <= 0) return fail(h, SPC_ERR_INVALID, "nsteps must be positive");
  if (!h->uploaded) return fail(h, SPC_ERR_STATE, "state not uploaded");
  if (h->injecting) return fail(h, SPC_ERR_STATE, "graph replay needs Philox noise");
  if (h->p.model == SPC_MODEL_VORTEX && !h->omega_set)
    return fail(h, SPC_ERR_STATE, "vortex model: natural frequencies not uploaded");
  SPC_TRY(set_device(h));
  if (!h->graph || h->graph_steps != nsteps || h->graph_dt != dt) {
    if (h->graph) {
      cudaGraphExecDestroy(h->graph);
      h->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    SPC_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = SPC_OK;
    for (int s = 0; s < nsteps && rc == SPC_OK; ++s) rc = enqueue_step(h, dt, s, nullptr);
    cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (rc != SPC_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return fail(h, SPC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      h->graph = nullptr;
      return fail(h, SPC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    }
    h->graph_steps = nsteps;
    h->graph_dt = dt;
  }
  SPC_TRY(write_step(h));
  SPC_CUDA(h, cudaGraphLaunch(h->graph, h->stream));
  double t = *t_inout;
  for (int s = 0; s < nsteps; ++s) t += dt;
  h->step += (uint64_t)nsteps;
  *t_inout = t;
  return SPC_OK;
}

int spc_get_step_counter(const spc_handle *h, uint64_t *out) {
  if (!h || !out) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  *out = h->step;
  return SPC_OK;
}

int spc_set_step_counter(spc_handle *h, uint64_t step) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  h->step = step;
  return SPC_OK;
}

int spc_inject_noise(spc_handle *h, const double *normals, int64_t count) {
  if (!h || (!normals && count > 0) || count < 0) return fail(h, SPC_ERR_INVALID, "bad argument");
  const int64_t per_step = (int64_t)noise_m(h->p) * h->n;
  if (per_step == 0) return fail(h, SPC_ERR_INVALID, "this stepper draws no noise");
  if (count % per_step) return fail(h, SPC_ERR_INVALID, "count must be a multiple of %lld", (long long)per_step);
  SPC_TRY(set_device(h));
  if (h->d_noise && h->noise_count < count) {
    SPC_CUDA(h, cudaStreamSynchronize(h->stream));
    auto it = std::find(h->allocs.begin(), h->allocs.end(), (void *)h->d_noise);
    if (it != h->allocs.end()) h->allocs.erase(it);
    cudaFree(h->d_noise);
    h->d_noise = nullptr;
  }
  if (!h->d_noise) SPC_TRY(dalloc(h, &h->d_noise, (size_t)std::max<int64_t>(count, 1)));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  SPC_CUDA(h, cudaMemcpy(h->d_noise, normals, (size_t)count * 8, cudaMemcpyHostToDevice));
  h->noise_count = count;
  h->noise_cursor = 0;
  h->injecting = true;
  return SPC_OK;
}

int spc_clear_noise(spc_handle *h) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  h->injecting = false;
  h->noise_cursor = h->noise_count = 0;
  return SPC_OK;
}

int spc_export_noise(spc_handle *h, uint64_t first_step, int32_t nsteps, double *out) {
  if (!h || !out || nsteps < 0) return fail(h, SPC_ERR_INVALID, "bad argument");
  const int m = noise_m(h->p);
  if (m == 0 || nsteps == 0) return SPC_OK;
  SPC_TRY(set_device(h));
  const size_t count = (size_t)nsteps * h->n * m;
  double *d = nullptr;
  SPC_CUDA(h, cudaMalloc(&d, count * 8));
  k_export_noise<<<blocks_for((long long)nsteps * h->n, 256), 256, 0, h->stream>>>(
      h->p.seed, h->p.system_id, first_step, nsteps, h->n, m, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, count * 8, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (e != cudaSuccess) return fail(h, SPC_ERR_CUDA, "export noise: %s", cudaGetErrorString(e));
  return SPC_OK;
}

int spc_rhs_rk(spc_handle *h, const double *k_prev, double k_coef, double dt, double *k_next) {
  if (!h || !k_prev || !k_next) return fail(h, SPC_ERR_INVALID, "NULL argument");
  if (!h->uploaded) return fail(h, SPC_ERR_STATE, "state not uploaded");
  SPC_TRY(set_device(h));
  KArgs &base = h->a;
  const size_t N = h->n;
  if (!h->scratch_k) {
    for (int q = 4; q < 6; ++q) {
      SPC_TRY(dalloc(h, &base.kx[q], N));
      SPC_TRY(dalloc(h, &base.ky[q], N));
      SPC_TRY(dalloc(h, &base.kphi[q], N));
    }
    h->scratch_k = true;
  }
  SPC_CUDA(h, cudaMemcpyAsync(h->aos, k_prev, 3 * N * 8, cudaMemcpyHostToDevice, h->stream));
  SPC_CUDA(h, cudaMemcpyAsync(h->aos + 3 * N, k_next, 3 * N * 8, cudaMemcpyHostToDevice, h->stream));
  k_aos_to_soa<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->aos, h->n, base.kx[4], base.ky[4], base.kphi[4]);
  k_aos_to_soa<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->aos + 3 * N, h->n, base.kx[5], base.ky[5],
                                                              base.kphi[5]);
  SPC_LAUNCHED(h);
  KArgs a = base;
  SPC_TRY(eval_stage(h, a, 1, 4, k_coef * dt));
  a.kq_out = 5;
  SPC_TRY(launch_pass(h, a, kKindSin, kEpiRkK));
  k_soa_to_aos<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(base.kx[5], base.ky[5], base.kphi[5], h->n, h->aos);
  SPC_LAUNCHED(h);
  SPC_CUDA(h, cudaMemcpyAsync(k_next, h->aos, 3 * N * 8, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPC_OK;
}

int spc_rhs_srk(spc_handle *h, double *derivative, double *additional) {
  if (!h || !derivative || !additional) return fail(h, SPC_ERR_INVALID, "NULL argument");
  if (!h->uploaded) return fail(h, SPC_ERR_STATE, "state not uploaded");
  SPC_TRY(set_device(h));
  const size_t N = h->n;
  KArgs a = h->a;
  a.out_d = h->aos;
  a.out_a = h->aos + 3 * N;
  SPC_TRY(eval_stage(h, a, 0, -1, 0.0));
  SPC_TRY(launch_pass(h, a, kKindSin, kEpiSrk1));
  SPC_TRY(launch_pass(h, a, kKindCos2, kEpiSrk2Out));
  SPC_CUDA(h, cudaMemcpyAsync(derivative, a.out_d, 3 * N * 8, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaMemcpyAsync(additional, a.out_a, 2 * N * 8, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPC_OK;
}

int spc_neighbours(spc_handle *h, int32_t *counts, int32_t *idx, int64_t cap, int64_t *total) {
  if (!h || !counts) return fail(h, SPC_ERR_INVALID, "NULL argument");
  if (!h->uploaded) return fail(h, SPC_ERR_STATE, "state not uploaded");
  SPC_TRY(set_device(h));
  const size_t N = h->n;
  KArgs a = h->a;
  int *d_cnt = (int *)h->aos;  // 12N doubles of staging: counts, offsets, list head
  a.out_cnt = d_cnt;
  SPC_TRY(eval_stage(h, a, 0, -1, 0.0));
  SPC_TRY(launch_pass(h, a, kKindNb, kEpiCount));
  SPC_CUDA(h, cudaMemcpyAsync(counts, d_cnt, N * 4, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<long long> off(N + 1, 0);
  for (size_t i = 0; i < N; ++i) off[i + 1] = off[i] + counts[i];
  if (total) *total = off[N];
  if (!idx) return SPC_OK;
  if (cap < off[N]) return fail(h, SPC_ERR_CAPACITY, "need %lld indices, cap %lld", off[N], (long long)cap);
  long long *d_off = nullptr;
  int *d_idx = nullptr;
  cudaError_t e = cudaMalloc(&d_off, (N + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&d_idx, std::max<long long>(off[N], 1) * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, off.data(), (N + 1) * 8, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) {
    a.list_off = d_off;
    a.list_idx = d_idx;
    int rc = launch_pass(h, a, kKindNb, kEpiCount);
    if (rc != SPC_OK) e = cudaErrorUnknown;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(idx, d_idx, off[N] * 4, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d_off);
  cudaFree(d_idx);
  if (e != cudaSuccess) return fail(h, SPC_ERR_CUDA, "neighbour list: %s", cudaGetErrorString(e));
  return SPC_OK;
}

int spc_order_params(spc_handle *h, double *R, double *psi, double *R_local) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  if (!h->uploaded) return fail(h, SPC_ERR_STATE, "state not uploaded");
  SPC_TRY(set_device(h));
  const size_t N = h->n;
  k_order_sum<<<h->order_blocks, 256, 0, h->stream>>>(h->a.phi, h->n, h->order_part);
  SPC_LAUNCHED(h);
  std::vector<double> part(2 * (size_t)h->order_blocks);
  SPC_CUDA(h, cudaMemcpyAsync(part.data(), h->order_part, part.size() * 8, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  double re = 0.0, im = 0.0;
  for (int b = 0; b < h->order_blocks; ++b) {
    re += part[2 * b];
    im += part[2 * b + 1];
  }
  re /= (double)N;
  im /= (double)N;
  if (R) *R = std::hypot(re, im);
  if (psi) *psi = std::atan2(im, re);
  if (R_local) {
    KArgs a = h->a;
    a.out_r = h->aos;
    SPC_TRY(eval_stage(h, a, 0, -1, 0.0));
    SPC_TRY(launch_pass(h, a, kKindNb, kEpiLocalOrder));
    std::vector<double> r(N);
    SPC_CUDA(h, cudaMemcpyAsync(r.data(), a.out_r, N * 8, cudaMemcpyDeviceToHost, h->stream));
    SPC_CUDA(h, cudaStreamSynchronize(h->stream));
    double acc = 0.0;
    for (size_t i = 0; i < N; ++i) acc += r[i];
    *R_local = acc / (double)N;
  }
  return SPC_OK;
}

int spc_diagnostics(spc_handle *h, int64_t *clamped_cells, int64_t *verlet_rebuilds, int64_t *error_word) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(set_device(h));
  unsigned long long c = 0;
  SPC_CUDA(h, cudaMemcpyAsync(&c, h->d_clamped, 8, cudaMemcpyDeviceToHost, h->stream));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  if (clamped_cells) *clamped_cells = (int64_t)c;
  if (verlet_rebuilds) *verlet_rebuilds = 0;
  if (error_word) *error_word = 0;
  return SPC_OK;
}

int spc_synchronize(spc_handle *h) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(set_device(h));
  SPC_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPC_OK;
}

void *spc_stream(spc_handle *h) { return h ? (void *)h->stream : nullptr; }

int spc_profile_steps(spc_handle *h, double dt, int32_t nsteps, double *out_ms, int32_t cap) {
  if (!h || !out_ms || cap < 6 || nsteps <= 0) return fail(h, SPC_ERR_INVALID, "bad argument");
  if (!h->uploaded) return fail(h, SPC_ERR_STATE, "state not uploaded");
  if (h->injecting) return fail(h, SPC_ERR_STATE, "profiling uses Philox noise");
  SPC_TRY(set_device(h));
  for (int e = 0; e < 6; ++e)
    if (!h->prof_ev[e]) SPC_CUDA(h, cudaEventCreate(&h->prof_ev[e]));
  double acc[6] = {0, 0, 0, 0, 0, 0};
  SPC_TRY(write_step(h));
  for (int s = 0; s < nsteps; ++s) {
    // phase marks: 0 start, 1 after stage, 2 after sort, 3 after gather,
    // 4 after the first pass, 5 end of step
    SPC_CUDA(h, cudaEventRecord(h->prof_ev[0], h->stream));
    h->profiling = true;
    int rc = enqueue_step(h, dt, s, nullptr);
    h->profiling = false;
    if (rc != SPC_OK) return rc;
    SPC_CUDA(h, cudaEventRecord(h->prof_ev[5], h->stream));
    SPC_CUDA(h, cudaEventSynchronize(h->prof_ev[5]));
    float ms[6] = {0, 0, 0, 0, 0, 0};
    for (int e = 1; e <= 5; ++e) SPC_CUDA(h, cudaEventElapsedTime(&ms[e], h->prof_ev[e - 1], h->prof_ev[e]));
    for (int e = 0; e < 5; ++e) acc[e] += ms[e + 1];
    float tot = 0.0f;
    SPC_CUDA(h, cudaEventElapsedTime(&tot, h->prof_ev[0], h->prof_ev[5]));
    acc[5] += tot;
  }
  h->step += (uint64_t)nsteps;
  for (int e = 0; e < 6; ++e) out_ms[e] = acc[e] / nsteps;
  return SPC_OK;
}

int spc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  if (!ctr || !key || !out) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  uint32_t *d = nullptr;
  cudaError_t e = cudaMalloc(&d, 16);
  if (e == cudaSuccess) {
    k_philox_kat<<<1, 1>>>(U4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1], d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d, 16, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "philox: %s", cudaGetErrorString(e));
  return SPC_OK;
}

int spc_alloc_pinned(size_t bytes, void **out) {
  if (!out) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_NOMEM, "cudaMallocHost: %s", cudaGetErrorString(e));
  return SPC_OK;
}

int spc_free_pinned(void *p) {
  if (p) cudaFreeHost(p);
  return SPC_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free SRK right-hand side.
//
// Some callers cannot call cudaMalloc at the point where they need a
// right-hand side: code that runs while another component owns every byte of
// device memory through its own pool, latency-critical loops where a
// cudaMalloc/cudaFree pair would synchronise the device, and hosts that must
// not grow their device footprint after start-up.  spc_rhs_srk_noalloc serves
// them: the caller passes device input and output buffers, and every
// intermediate array (cell keys, the radix sort's buffers and histograms, the
// cell table, the cell-order copies) lives in one file-scope __device__ array
// of fixed size, resident on every GPU that loads this library until the
// process exits.
namespace {

constexpr int kNoAllocMaxN = 8192;       // particles per call
constexpr int kNoAllocMaxCells = 16384;  // cells (nc * nc) per call
constexpr int kNoAllocMaxTiles = (kNoAllocMaxN + kSortTile - 1) / kSortTile;

constexpr size_t na_round(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kNaD = na_round(8ull * kNoAllocMaxN);   // one double per particle
constexpr size_t kNaF = na_round(4ull * kNoAllocMaxN);   // one 32-bit value per particle
constexpr size_t kNaF2 = na_round(8ull * kNoAllocMaxN);  // one float2 per particle
constexpr size_t kNaCells = na_round(4ull * (kNoAllocMaxCells + 1));
constexpr size_t kNaHist = na_round(4ull * (1u << 11) * kNoAllocMaxTiles);
// x y phi | st_x st_y st_phi | sx sy sphi | dphi_s  (10 double arrays)
// keys vals keys_alt vals_alt pidx cnt_s dphi_f    (7 32-bit arrays)
// fxy cs (2 float2 arrays) | cell_start | hist | clamped counter
constexpr size_t kNoAllocBytes = 10 * kNaD + 7 * kNaF + 2 * kNaF2 + kNaCells + kNaHist + 256;

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
char *g_noalloc_base[kNoAllocMaxDevices] = {};

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

// Device address of g_noalloc_scratch on the current device.  In host code
// the symbol name is only a stand-in, so the address is looked up once per
// device with that device current and cached.
int noalloc_scratch(char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(nullptr, SPC_ERR_INVALID, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_base[dev]) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(nullptr, SPC_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_noalloc_base[dev] = (char *)ptr;
  }
  *out = g_noalloc_base[dev];
  return SPC_OK;
}

}  // namespace

extern "C" int spc_rhs_srk_noalloc(const spc_params *p, int32_t n, const double *d_state,
                                   double *d_derivative, double *d_additional, void *stream) {
  int rc = validate(p, n, nullptr);
  if (rc) return rc;
  if (!d_state || !d_derivative || !d_additional)
    return fail(nullptr, SPC_ERR_INVALID, "NULL device buffer");
  if (n > kNoAllocMaxN)
    return fail(nullptr, SPC_ERR_CAPACITY, "spc_rhs_srk_noalloc: n = %d exceeds its maximum of %d particles",
                n, kNoAllocMaxN);
  const bool allpairs = !(p->rho <= 0.25 * p->L);
  const int nc = allpairs ? 1 : std::max(1, (int)(p->L / p->rho));
  if ((long long)nc * nc > kNoAllocMaxCells)
    return fail(nullptr, SPC_ERR_CAPACITY, "spc_rhs_srk_noalloc: %d x %d cells exceed its maximum of %d cells",
                nc, nc, kNoAllocMaxCells);
  char *base = nullptr;
  rc = noalloc_scratch(&base);
  if (rc) return rc;

  spc_handle h;  // a view: every pointer below is inside the static scratch
  h.p = *p;
  h.n = n;
  h.stream = (cudaStream_t)stream;
  SysConst &sc = h.sc;
  sc.n = n;
  sc.L = p->L;
  sc.rL = 1.0 / p->L;
  sc.rho2 = p->rho * p->rho;
  sc.v0 = p->v0;
  sc.sigma = p->sigma;
  sc.alpha = p->alpha;
  sc.D = p->D_phi;
  sc.allpairs = allpairs;
  sc.nc = nc;
  sc.ncell = nc * nc;
  sc.cell = p->L / nc;
  sc.cell_f = (float)sc.cell;
  sc.lo2 = (float)(sc.rho2 * (1.0 - 3e-5));
  sc.hi2 = (float)(sc.rho2 * (1.0 + 3e-5));
  sc.exact_all = (p->flags & SPC_FLAG_EXACT_ALL) ? 1 : 0;
  sc.L_pow2 = is_pow2(p->L);

  KArgs &a = h.a;
  a.sc = sc;
  char *cur = base;
  auto take = [&](size_t bytes) {
    char *r = cur;
    cur += bytes;
    return (void *)r;
  };
  a.x = (double *)take(kNaD);
  a.y = (double *)take(kNaD);
  a.phi = (double *)take(kNaD);
  a.st_x = (double *)take(kNaD);
  a.st_y = (double *)take(kNaD);
  a.st_phi = (double *)take(kNaD);
  a.sx = (double *)take(kNaD);
  a.sy = (double *)take(kNaD);
  a.sphi = (double *)take(kNaD);
  a.dphi_s = (double *)take(kNaD);
  a.keys = (uint32_t *)take(kNaF);
  a.vals = (uint32_t *)take(kNaF);
  h.keys_alt = (uint32_t *)take(kNaF);
  h.vals_alt = (uint32_t *)take(kNaF);
  a.pidx = (int *)take(kNaF);
  a.cnt_s = (int *)take(kNaF);
  a.dphi_f = (float *)take(kNaF);
  a.fxy = (float2 *)take(kNaF2);
  a.cs = (float2 *)take(kNaF2);
  a.cell_start = (int *)take(kNaCells);
  h.hist = (uint32_t *)take(kNaHist);
  unsigned long long *clamped = (unsigned long long *)take(256);
  a.clamped = clamped;
  a.omega = nullptr;
  a.out_d = d_derivative;
  a.out_a = d_additional;
  h.ntiles = (n + kSortTile - 1) / kSortTile;
  int bits = 1;
  while (bits < 31 && (1u << bits) < (unsigned)sc.ncell) ++bits;
  h.radix_bits = (bits <= 11) ? bits : 8;
  h.sort_passes = (bits + h.radix_bits - 1) / h.radix_bits;
  a.hist = h.hist;
  a.hist_len = (1 << h.radix_bits) * h.ntiles;

  cudaError_t e = set_kernel_attributes();
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "kernel attributes: %s", cudaGetErrorString(e));
  // the scratch keeps the previous call's contents: the clamp counter and the
  // radix histogram table are accumulated into, so they are cleared here
  e = cudaMemsetAsync(clamped, 0, 8, h.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(h.hist, 0, (size_t)a.hist_len * 4, h.stream);
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "clear scratch: %s", cudaGetErrorString(e));
  k_aos_to_soa<<<blocks_for(n, 256), 256, 0, h.stream>>>(d_state, n, a.x, a.y, a.phi);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
  KArgs run = a;
  rc = eval_stage(&h, run, 0, -1, 0.0);
  if (rc == SPC_OK) rc = launch_pass(&h, run, kKindSin, kEpiSrk1);
  if (rc == SPC_OK) rc = launch_pass(&h, run, kKindCos2, kEpiSrk2Out);
  return rc;
}
