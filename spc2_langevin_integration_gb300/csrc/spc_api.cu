// C-ABI implementation (include/spc_gb300.h).  A single-system handle is an
// engine (spc_engine.cuh) holding one system; a batch holds many and runs
// them in the same launches.  No CPU fallback: every entry point that
// computes launches the kernels of spc_kernels.cuh / spc_tile.cuh / spc_sort.cuh.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/spc_gb300.h"
#include "spc_engine.cuh"

using namespace spc;

struct spc_handle {
  Engine e;
  spc_params p{};
  int n = 0;
  int slot = 0;
  bool uploaded = false;
};

struct spc_batch {
  Engine e;
};

namespace {

int hfail(spc_handle *h, int code, const char *msg) {
  return fail(h ? &h->e : nullptr, code, "%s", msg);
}

// Evaluations outside a step loop (right-hand sides, diagnostics) run with a
// budget of one step so that k_next is written, and close with budget 0.
int open_eval(Engine *e, int budget) {
  k_begin_call<<<blocks_for(e->nsys, 128), 128, 0, e->stream>>>(e->d_sys, e->nsys, budget);
  SPC_LAUNCHED(e);
  return SPC_OK;
}

int check_ready(spc_handle *h) {
  if (!h->uploaded) return fail(&h->e, SPC_ERR_STATE, "state not uploaded");
  if (h->p.model == SPC_MODEL_VORTEX && !h->e.slots[h->slot].omega_set)
    return fail(&h->e, SPC_ERR_STATE, "vortex model: natural frequencies not uploaded");
  return SPC_OK;
}

// ---------------------------------------------------------------------------
// observed run loop (spc_run)

// Ring buffers of `doubles` each (device + pinned host), the copy stream and
// its events, created or grown on demand.
int run_pipe_reserve(Engine *e, size_t doubles) {
  Engine::RunPipe &r = e->run;
  if (!r.copy) {
    SPC_CUDA(e, cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
      SPC_CUDA(e, cudaEventCreateWithFlags(&r.computed[b], cudaEventDisableTiming));
      SPC_CUDA(e, cudaEventCreateWithFlags(&r.copied[b], cudaEventDisableTiming));
    }
  }
  doubles = std::max<size_t>(doubles, 1);
  if (r.ring_doubles >= doubles) return SPC_OK;
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(r.copy));
  drop_graph(e);  // the captured chunks write the old rings
  for (int b = 0; b < 2; ++b) {
    if (r.d_ring[b]) {
      auto it = std::find(e->allocs.begin(), e->allocs.end(), (void *)r.d_ring[b]);
      if (it != e->allocs.end()) e->allocs.erase(it);
      cudaFree(r.d_ring[b]);
      r.d_ring[b] = nullptr;
    }
    if (r.h_ring[b]) cudaFreeHost(r.h_ring[b]);
    r.h_ring[b] = nullptr;
  }
  r.ring_doubles = 0;
  for (int b = 0; b < 2; ++b) {
    SPC_TRY(dalloc(e, &r.d_ring[b], doubles));
    cudaError_t ce = cudaHostAlloc((void **)&r.h_ring[b], doubles * 8, cudaHostAllocDefault);
    if (ce != cudaSuccess) {
      r.h_ring[b] = nullptr;
      return fail(e, SPC_ERR_NOMEM, "cudaHostAlloc(%zu bytes): %s", doubles * 8, cudaGetErrorString(ce));
    }
  }
  r.ring_doubles = doubles;
  return SPC_OK;
}

// Enqueue one chunk of len steps, with a snapshot into ring b after every
// step whose pattern entry is set.
int run_enqueue_chunk(spc_handle *h, double dt, int len, const uint8_t *pat, int b,
                      const double *noise, long long per_step) {
  Engine *e = &h->e;
  const SysHost &sh = e->slots[h->slot];
  const size_t snap = 3 * (size_t)h->n;
  k_begin_call<<<blocks_for(e->nsys, 128), 128, 0, e->stream>>>(e->d_sys, e->nsys, len);
  SPC_LAUNCHED(e);
  int k = 0;
  for (int s = 0; s < len; ++s) {
    SPC_TRY(enqueue_step(e, dt, s, noise ? noise + (long long)s * per_step : nullptr));
    if (pat[s]) {
      k_soa_to_aos<<<blocks_for(h->n, 256), 256, 0, e->stream>>>(
          e->a.x + sh.pool_p0, e->a.y + sh.pool_p0, e->a.phi + sh.pool_p0, h->n,
          e->run.d_ring[b] + (size_t)k * snap);
      SPC_LAUNCHED(e);
      ++k;
    }
  }
  k_end_call<<<blocks_for(e->nsys, 128), 128, 0, e->stream>>>(e->d_sys, e->nsys);
  SPC_LAUNCHED(e);
  return SPC_OK;
}

// Capture the two chunk graphs (one per ring) for chunks of G steps.
int run_capture(spc_handle *h, double dt, int G, const std::vector<uint8_t> &pat) {
  Engine *e = &h->e;
  Engine::RunPipe &r = e->run;
  if (r.graph[0] && r.graph[1] && r.steps == G && r.dt == dt && r.pattern == pat) return SPC_OK;
  for (cudaGraphExec_t &g : r.graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (int b = 0; b < 2; ++b) {
    cudaGraph_t g = nullptr;
    SPC_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = run_enqueue_chunk(h, dt, G, pat.data(), b, nullptr, 0);
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (rc != SPC_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return fail(e, SPC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    r.graph_nodes = 0;
    cudaGraphGetNodes(g, nullptr, &r.graph_nodes);
    ce = cudaGraphInstantiate(&r.graph[b], g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      r.graph[b] = nullptr;
      return fail(e, SPC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    }
  }
  r.steps = G;
  r.dt = dt;
  r.pattern = pat;
  return SPC_OK;
}

bool batch_slot_ok(spc_batch *b, int slot) {
  return slot >= 0 && slot < b->e.sys_cap && b->e.slots[slot].used;
}

}  // namespace

// ===========================================================================
extern "C" {

int spc_abi_version(void) { return SPC_ABI_VERSION; }

const char *spc_last_error(const spc_handle *h) {
  if (h) return h->e.err.c_str();
  std::lock_guard<std::mutex> lk(err_mutex());
  return global_error().c_str();
}

int spc_destroy(spc_handle *h) {
  if (!h) return SPC_OK;
  engine_free(&h->e);
  delete h;
  return SPC_OK;
}

int spc_create(const spc_params *p, int32_t n, spc_handle **out) {
  if (!out) return fail(nullptr, SPC_ERR_INVALID, "out is NULL");
  *out = nullptr;
  std::string why;
  int rc = validate_params(p, n, why);
  if (rc) return fail(nullptr, rc, "%s", why.c_str());
  spc_handle *h = new spc_handle();
  h->p = *p;
  h->n = n;
  const SysConst sc = make_sysconst(*p, n);
  rc = engine_init(&h->e, p->stepper, p->precision, n, 1, sc.allpairs ? 1 : sc.ncell);
  if (rc == SPC_OK && sc.vR > 0) {
    // rows of about pi r_max^2 n / L^2 entries: room for twice that (and for
    // eight standard deviations of a uniform layout), at most 1024
    const double rmax = p->rho + p->skin;
    const double mean = 3.141592653589793 * rmax * rmax * (double)n / (p->L * p->L);
    const double want = std::max(2.0 * mean, mean + 8.0 * std::sqrt(mean)) + 64.0;
    rc = engine_init_verlet(&h->e, ((int)want + 31) / 32 * 32);
  }
  // (cells dense enough for the cell-tile kernel by default: the warp-per-cell
  // kernel of sparse cells keeps no cosines)
  if (rc == SPC_OK && p->model != SPC_MODEL_VORTEX_ARRAYS && p->stepper == SPC_STEPPER_SRK &&
      p->precision == SPC_PRECISION_FP64 && p->neighbour == SPC_NEIGHBOUR_CELL && !sc.allpairs &&
      (double)n / (double)sc.ncell >= kSparseBelowDefault) {
    // accepted pairs: about pi rho^2 n / L^2 per particle
    const double mean = 3.141592653589793 * p->rho * p->rho * (double)n / (p->L * p->L);
    const double want = std::max(2.0 * mean, mean + 8.0 * std::sqrt(mean)) + 64.0;
    rc = engine_init_tile_cos(&h->e, ((int)std::min(want, (double)n) + 31) / 32 * 32);
  }
  if (rc == SPC_OK && p->model == SPC_MODEL_VORTEX_ARRAYS && p->stepper == SPC_STEPPER_SRK) {
    // pairs within rho: about pi rho^2 n / L^2 per particle
    const double mean = 3.141592653589793 * p->rho * p->rho * (double)n / (p->L * p->L);
    const double want = std::max(2.0 * mean, mean + 8.0 * std::sqrt(mean)) + 64.0;
    rc = engine_init_va_cache(&h->e, ((int)std::min(want, (double)n) + 31) / 32 * 32);
  }
  if (rc == SPC_OK) rc = engine_admit(&h->e, *p, n, -1, &h->slot);
  if (rc == SPC_OK) {
    Engine &e = h->e;
    cudaError_t ce = cudaMemsetAsync(e.a.x, 0, (size_t)n * 8, e.stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(e.a.y, 0, (size_t)n * 8, e.stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(e.a.phi, 0, (size_t)n * 8, e.stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e.stream);
    if (ce != cudaSuccess) rc = fail(&e, SPC_ERR_CUDA, "init: %s", cudaGetErrorString(ce));
  }
  if (rc != SPC_OK) {
    std::string msg = h->e.err;
    spc_destroy(h);
    fail(nullptr, rc, "%s", msg.c_str());
    return rc;
  }
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
  if (!h || !aos3n) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(engine_set_device(&h->e));
  SPC_TRY(engine_upload(&h->e, h->slot, aos3n));
  h->uploaded = true;
  return SPC_OK;
}

int spc_download_state(spc_handle *h, double *aos3n) {
  if (!h || !aos3n) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(engine_set_device(&h->e));
  return engine_download(&h->e, h->slot, aos3n);
}

int spc_upload_omega(spc_handle *h, const double *omega) {
  if (!h || !omega) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(engine_set_device(&h->e));
  return engine_upload_omega(&h->e, h->slot, omega);
}

int spc_download_rk4_buffers(spc_handle *h, double *out12n) {
  if (!h || !out12n) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  if (h->p.stepper != SPC_STEPPER_RK4) return hfail(h, SPC_ERR_STATE, "not an RK4 system");
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  const size_t N = h->n;
  for (int q = 0; q < 4; ++q) {
    k_soa_to_aos<<<blocks_for(h->n, 256), 256, 0, e->stream>>>(e->a.kx[q], e->a.ky[q], e->a.kphi[q], h->n,
                                                               e->aos + q * 3 * N);
    SPC_LAUNCHED(e);
  }
  SPC_CUDA(e, cudaMemcpyAsync(out12n, e->aos, 12 * N * 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  return SPC_OK;
}

int spc_upload_rk4_buffers(spc_handle *h, const double *in12n) {
  if (!h || !in12n) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  if (h->p.stepper != SPC_STEPPER_RK4) return hfail(h, SPC_ERR_STATE, "not an RK4 system");
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  const size_t N = h->n;
  SPC_CUDA(e, cudaMemcpyAsync(e->aos, in12n, 12 * N * 8, cudaMemcpyHostToDevice, e->stream));
  for (int q = 0; q < 4; ++q) {
    k_aos_to_soa<<<blocks_for(h->n, 256), 256, 0, e->stream>>>(e->aos + q * 3 * N, h->n, e->a.kx[q],
                                                               e->a.ky[q], e->a.kphi[q]);
    SPC_LAUNCHED(e);
  }
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  return SPC_OK;
}

int spc_noise_per_particle(const spc_handle *h) { return h ? noise_per_particle(h->p.stepper) : 0; }

int spc_step(spc_handle *h, double *t_inout, double dt, int32_t nsteps) {
  if (!h || !t_inout) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  if (nsteps < 0) return hfail(h, SPC_ERR_INVALID, "nsteps must be >= 0");
  SPC_TRY(check_ready(h));
  Engine *e = &h->e;
  const long long per_step = (long long)noise_per_particle(h->p.stepper) * h->n;
  const double *noise = nullptr;
  if (e->injecting && per_step > 0) {
    if (e->noise_cursor + per_step * nsteps > e->noise_count)
      return fail(e, SPC_ERR_NOISE, "injected noise: %lld normals left, %lld needed",
                  e->noise_count - e->noise_cursor, per_step * nsteps);
    noise = e->d_noise + e->noise_cursor;
  }
  SPC_TRY(engine_steps(e, dt, nsteps, false, noise, per_step));
  if (noise) e->noise_cursor += per_step * nsteps;
  double t = *t_inout;
  for (int s = 0; s < nsteps; ++s) t += dt;  // SimulationEngine.cpp:151
  *t_inout = t;
  return SPC_OK;
}

int spc_step_graph(spc_handle *h, double *t_inout, double dt, int32_t nsteps) {
  if (!h || !t_inout) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  if (nsteps <= 0) return hfail(h, SPC_ERR_INVALID, "nsteps must be positive");
  SPC_TRY(check_ready(h));
  if (h->e.injecting) return fail(&h->e, SPC_ERR_STATE, "graph replay needs Philox noise");
  SPC_TRY(engine_steps(&h->e, dt, nsteps, true, nullptr, 0));
  double t = *t_inout;
  for (int s = 0; s < nsteps; ++s) t += dt;
  *t_inout = t;
  return SPC_OK;
}

int spc_prepare_graph(spc_handle *h, double dt, int32_t nsteps) {
  if (!h) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  if (nsteps <= 0) return hfail(h, SPC_ERR_INVALID, "nsteps must be positive");
  SPC_TRY(check_ready(h));
  if (h->e.injecting) return fail(&h->e, SPC_ERR_STATE, "graph replay needs Philox noise");
  return engine_prepare_graph(&h->e, dt, nsteps);
}

int spc_run(spc_handle *h, double *t_inout, double dt, int64_t nsteps, int32_t period,
            const uint8_t *observe, spc_observe_fn fn, void *user, int64_t *steps_done) {
  if (steps_done) *steps_done = 0;
  if (!h || !t_inout) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  if (nsteps < 0) return hfail(h, SPC_ERR_INVALID, "nsteps must be >= 0");
  if (period < 1) return hfail(h, SPC_ERR_INVALID, "period must be >= 1");
  if (fn && !observe) return hfail(h, SPC_ERR_INVALID, "observe is NULL");
  SPC_TRY(check_ready(h));
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  const long long per_step = (long long)noise_per_particle(h->p.stepper) * h->n;
  const bool inject = e->injecting && per_step > 0;
  if (inject && e->noise_cursor + per_step * nsteps > e->noise_count)
    return fail(e, SPC_ERR_NOISE, "injected noise: %lld normals left, %lld needed",
                e->noise_count - e->noise_cursor, per_step * (long long)nsteps);
  if (nsteps == 0) return SPC_OK;
  // chunks of G = m periods (about 64 steps) whose snapshots fit rings of 512 MB
  const size_t snap = 3 * (size_t)h->n;
  int obs_per_period = 0;
  if (fn)
    for (int j = 0; j < period; ++j) obs_per_period += observe[j] != 0;
  long long m = std::max(1, 64 / period);
  const size_t ring_cap = ((size_t)512 << 20) / 8;
  while (m > 1 && (size_t)(obs_per_period * m) * snap > ring_cap) --m;
  const long long G = std::min<long long>(period * m, nsteps);
  std::vector<uint8_t> full((size_t)G);
  int obs_chunk = 0;
  for (long long s = 0; s < G; ++s) {
    full[(size_t)s] = fn && observe[(s + 1) % period] ? 1 : 0;
    obs_chunk += full[(size_t)s];
  }
  SPC_TRY(run_pipe_reserve(e, (size_t)obs_chunk * snap));
  SPC_TRY(engine_layout(e));
  SPC_TRY(verlet_prepare(e));
  const bool use_graph = !inject && G <= 1024;
  if (use_graph) SPC_TRY(run_capture(h, dt, (int)G, full));
  Engine::RunPipe &r = e->run;
  struct Chunk {
    long long first, len;
    int b, nobs;
  };
  bool have_prev = false, stop = false;
  Chunk prev{};
  long long done = 0;
  double t_cb = *t_inout;
  int rc = SPC_OK;
  std::vector<uint8_t> pat;
  for (int c = 0; rc == SPC_OK; ++c) {
    Chunk cur{};
    const bool more = done < nsteps && !stop;
    if (more) {
      cur.first = done;
      cur.len = std::min<long long>(G, nsteps - done);
      cur.b = c & 1;
      pat.assign((size_t)cur.len, 0);
      cur.nobs = 0;
      for (long long s = 0; s < cur.len; ++s) {
        pat[(size_t)s] = fn && observe[(done + s + 1) % period] ? 1 : 0;
        cur.nobs += pat[(size_t)s];
      }
      // the ring's previous copy (chunk c - 2) completed before its callbacks
      const double *noise = inject ? e->d_noise + e->noise_cursor : nullptr;
      if (use_graph && cur.len == G) {
        const cudaError_t ce = cudaGraphLaunch(r.graph[cur.b], e->stream);
        if (ce != cudaSuccess) rc = fail(e, SPC_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ce));
      } else {
        rc = run_enqueue_chunk(h, dt, (int)cur.len, pat.data(), cur.b, noise, per_step);
      }
      if (rc != SPC_OK) break;
      mirror_call(e, (int)cur.len);
      if (inject) e->noise_cursor += per_step * cur.len;
      if (cur.nobs > 0) {
        cudaError_t ce = cudaEventRecord(r.computed[cur.b], e->stream);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(r.copy, r.computed[cur.b], 0);
        if (ce == cudaSuccess)
          ce = cudaMemcpyAsync(r.h_ring[cur.b], r.d_ring[cur.b], (size_t)cur.nobs * snap * 8,
                               cudaMemcpyDeviceToHost, r.copy);
        if (ce == cudaSuccess) ce = cudaEventRecord(r.copied[cur.b], r.copy);
        if (ce != cudaSuccess) {
          rc = fail(e, SPC_ERR_CUDA, "snapshot copy: %s", cudaGetErrorString(ce));
          break;
        }
      }
      done += cur.len;
    }
    if (have_prev) {
      // the previous chunk's snapshots, while the device runs this one
      if (prev.nobs > 0) {
        const cudaError_t ce = cudaEventSynchronize(r.copied[prev.b]);
        if (ce != cudaSuccess) {
          rc = fail(e, SPC_ERR_CUDA, "snapshot copy: %s", cudaGetErrorString(ce));
          break;
        }
      }
      int k = 0;
      for (long long s = 0; s < prev.len; ++s) {
        t_cb += dt;
        const long long step = prev.first + s + 1;
        if (fn && observe[step % period]) {
          if (!stop && fn(user, step, t_cb, r.h_ring[prev.b] + (size_t)k * snap) != 0) stop = true;
          ++k;
        }
      }
    }
    if (!more) break;
    prev = cur;
    have_prev = true;
  }
  // the state has advanced by every enqueued step
  cudaError_t ce = cudaStreamSynchronize(e->stream);
  if (ce == cudaSuccess && r.copy) ce = cudaStreamSynchronize(r.copy);
  if (rc == SPC_OK && ce != cudaSuccess) rc = fail(e, SPC_ERR_CUDA, "run: %s", cudaGetErrorString(ce));
  double t = *t_inout;
  for (long long s = 0; s < done; ++s) t += dt;  // SimulationEngine.cpp:151
  *t_inout = t;
  if (steps_done) *steps_done = done;
  return rc;
}

int spc_get_step_counter(const spc_handle *h, uint64_t *out) {
  if (!h || !out) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  *out = h->e.slots[h->slot].step;
  return SPC_OK;
}

int spc_set_step_counter(spc_handle *h, uint64_t step) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  engine_set_step(&h->e, h->slot, step);
  return SPC_OK;
}

int spc_inject_noise(spc_handle *h, const double *normals, int64_t count) {
  if (!h || (!normals && count > 0) || count < 0) return hfail(h, SPC_ERR_INVALID, "bad argument");
  Engine *e = &h->e;
  const long long per_step = (long long)noise_per_particle(h->p.stepper) * h->n;
  if (per_step == 0) return fail(e, SPC_ERR_INVALID, "this stepper draws no noise");
  if (count % per_step) return fail(e, SPC_ERR_INVALID, "count must be a multiple of %lld", per_step);
  SPC_TRY(engine_set_device(e));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  if (e->d_noise && e->noise_count < count) {
    auto it = std::find(e->allocs.begin(), e->allocs.end(), (void *)e->d_noise);
    if (it != e->allocs.end()) e->allocs.erase(it);
    cudaFree(e->d_noise);
    e->d_noise = nullptr;
  }
  if (!e->d_noise) SPC_TRY(dalloc(e, &e->d_noise, (size_t)std::max<int64_t>(count, 1)));
  SPC_CUDA(e, cudaMemcpy(e->d_noise, normals, (size_t)count * 8, cudaMemcpyHostToDevice));
  e->noise_count = count;
  e->noise_cursor = 0;
  e->injecting = true;
  return SPC_OK;
}

int spc_clear_noise(spc_handle *h) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  h->e.injecting = false;
  h->e.noise_cursor = h->e.noise_count = 0;
  return SPC_OK;
}

int spc_export_noise(spc_handle *h, uint64_t first_step, int32_t nsteps, double *out) {
  if (!h || !out || nsteps < 0) return hfail(h, SPC_ERR_INVALID, "bad argument");
  const int m = noise_per_particle(h->p.stepper);
  if (m == 0 || nsteps == 0) return SPC_OK;
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  const size_t count = (size_t)nsteps * h->n * m;
  double *d = nullptr;
  SPC_CUDA(e, cudaMalloc(&d, count * 8));
  k_export_noise<<<blocks_for((long long)nsteps * h->n, 256), 256, 0, e->stream>>>(
      h->p.seed, h->p.system_id, first_step, nsteps, h->n, m, d);
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(out, d, count * 8, cudaMemcpyDeviceToHost, e->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
  cudaFree(d);
  if (ce != cudaSuccess) return fail(e, SPC_ERR_CUDA, "export noise: %s", cudaGetErrorString(ce));
  return SPC_OK;
}

int spc_rhs_rk(spc_handle *h, const double *k_prev, double k_coef, double dt, double *k_next) {
  if (!h || !k_prev || !k_next) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(check_ready(h));
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  KArgs &base = e->a;
  const size_t N = h->n;
  if (!e->scratch_k) {
    for (int q = 4; q < 6; ++q) {
      SPC_TRY(dalloc(e, &base.kx[q], N));
      SPC_TRY(dalloc(e, &base.ky[q], N));
      SPC_TRY(dalloc(e, &base.kphi[q], N));
    }
    e->scratch_k = true;
  }
  SPC_CUDA(e, cudaMemcpyAsync(e->aos, k_prev, 3 * N * 8, cudaMemcpyHostToDevice, e->stream));
  SPC_CUDA(e, cudaMemcpyAsync(e->aos + 3 * N, k_next, 3 * N * 8, cudaMemcpyHostToDevice, e->stream));
  k_aos_to_soa<<<blocks_for(h->n, 256), 256, 0, e->stream>>>(e->aos, h->n, base.kx[4], base.ky[4], base.kphi[4]);
  k_aos_to_soa<<<blocks_for(h->n, 256), 256, 0, e->stream>>>(e->aos + 3 * N, h->n, base.kx[5], base.ky[5],
                                                             base.kphi[5]);
  SPC_LAUNCHED(e);
  KArgs a = base;
  a.dt = dt;
  a.sdt = std::sqrt(dt);
  SPC_TRY(verlet_prepare(e));
  SPC_TRY(open_eval(e, 1));
  SPC_TRY(eval_stage(e, a, 1, 4, k_coef * dt));
  a.kq_out = 5;
  SPC_TRY(launch_pass(e, a, kKindSin, kEpiRkK));
  SPC_TRY(open_eval(e, 0));
  k_soa_to_aos<<<blocks_for(h->n, 256), 256, 0, e->stream>>>(base.kx[5], base.ky[5], base.kphi[5], h->n, e->aos);
  SPC_LAUNCHED(e);
  SPC_CUDA(e, cudaMemcpyAsync(k_next, e->aos, 3 * N * 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  return SPC_OK;
}

int spc_rhs_srk(spc_handle *h, double *derivative, double *additional) {
  if (!h || !derivative || !additional) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(check_ready(h));
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  const size_t N = h->n;
  KArgs a = e->a;
  a.out_d = e->aos;
  a.out_a = e->aos + 3 * N;
  SPC_TRY(verlet_prepare(e));
  SPC_TRY(eval_stage(e, a, 0, -1, 0.0));
  SPC_TRY(launch_pass(e, a, kKindSin, kEpiSrk1));
  SPC_TRY(launch_pass(e, a, kKindCos2, kEpiSrk2Out));
  SPC_CUDA(e, cudaMemcpyAsync(derivative, a.out_d, 3 * N * 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaMemcpyAsync(additional, a.out_a, 2 * N * 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  return SPC_OK;
}

int spc_neighbours(spc_handle *h, int32_t *counts, int32_t *idx, int64_t cap, int64_t *total) {
  if (!h || !counts) return hfail(h, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(check_ready(h));
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  const size_t N = h->n;
  KArgs a = e->a;
  int *d_cnt = (int *)e->aos;
  a.out_cnt = d_cnt;
  SPC_TRY(eval_stage(e, a, 0, -1, 0.0, false));
  SPC_TRY(launch_pass(e, a, kKindNb, kEpiCount));
  SPC_CUDA(e, cudaMemcpyAsync(counts, d_cnt, N * 4, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  std::vector<long long> off(N + 1, 0);
  for (size_t i = 0; i < N; ++i) off[i + 1] = off[i] + counts[i];
  if (total) *total = off[N];
  if (!idx) return SPC_OK;
  if (cap < off[N]) return fail(e, SPC_ERR_CAPACITY, "need %lld indices, cap %lld", off[N], (long long)cap);
  long long *d_off = nullptr;
  int *d_idx = nullptr;
  cudaError_t ce = cudaMalloc(&d_off, (N + 1) * 8);
  if (ce == cudaSuccess) ce = cudaMalloc(&d_idx, std::max<long long>(off[N], 1) * 4);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_off, off.data(), (N + 1) * 8, cudaMemcpyHostToDevice, e->stream);
  if (ce == cudaSuccess) {
    a.list_off = d_off;
    a.list_idx = d_idx;
    if (launch_pass(e, a, kKindNb, kEpiCount) != SPC_OK) ce = cudaErrorUnknown;
  }
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(idx, d_idx, off[N] * 4, cudaMemcpyDeviceToHost, e->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
  cudaFree(d_off);
  cudaFree(d_idx);
  if (ce != cudaSuccess) return fail(e, SPC_ERR_CUDA, "neighbour list: %s", cudaGetErrorString(ce));
  return SPC_OK;
}

int spc_order_params(spc_handle *h, double *R, double *psi, double *R_local) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(check_ready(h));
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  SPC_TRY(engine_layout(e));
  SPC_TRY(engine_order_global(e, h->slot, R, psi));
  if (R_local) {
    const size_t N = h->n;
    KArgs a = e->a;
    a.out_r = e->aos;
    SPC_TRY(eval_stage(e, a, 0, -1, 0.0, false));
    SPC_TRY(launch_pass(e, a, kKindNb, kEpiLocalOrder));
    std::vector<double> r(N);
    SPC_CUDA(e, cudaMemcpyAsync(r.data(), a.out_r, N * 8, cudaMemcpyDeviceToHost, e->stream));
    SPC_CUDA(e, cudaStreamSynchronize(e->stream));
    double acc = 0.0;
    for (size_t i = 0; i < N; ++i) acc += r[i];
    *R_local = acc / (double)N;
  }
  return SPC_OK;
}

int spc_diagnostics(spc_handle *h, int64_t *clamped_cells, int64_t *verlet_rebuilds, int64_t *error_word) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  Engine *e = &h->e;
  SPC_TRY(engine_set_device(e));
  unsigned long long c = 0;
  SPC_CUDA(e, cudaMemcpyAsync(&c, e->d_clamped, 8, cudaMemcpyDeviceToHost, e->stream));
  SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  if (clamped_cells) *clamped_cells = (int64_t)c;
  unsigned long long vb = 0;
  if (e->verlet) {
    SPC_CUDA(e, cudaMemcpyAsync(&vb, e->vrebuilds, 8, cudaMemcpyDeviceToHost, e->stream));
    SPC_CUDA(e, cudaStreamSynchronize(e->stream));
  }
  if (verlet_rebuilds) *verlet_rebuilds = (int64_t)vb;
  if (error_word) *error_word = 0;
  return SPC_OK;
}

int spc_synchronize(spc_handle *h) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(engine_set_device(&h->e));
  SPC_CUDA(&h->e, cudaStreamSynchronize(h->e.stream));
  return SPC_OK;
}

void *spc_stream(spc_handle *h) { return h ? (void *)h->e.stream : nullptr; }

int spc_run_graph_nodes(const spc_handle *h, int64_t *nodes, int32_t *steps) {
  if (!h || !nodes) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  const bool have = h->e.run.graph[0] != nullptr;
  *nodes = have ? (int64_t)h->e.run.graph_nodes : 0;
  if (steps) *steps = have ? h->e.run.steps : 0;
  return SPC_OK;
}

int spc_graph_nodes(const spc_handle *h, int64_t *nodes) {
  if (!h || !nodes) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  *nodes = h->e.graph ? (int64_t)h->e.graph_nodes : 0;
  return SPC_OK;
}

int spc_profile_steps(spc_handle *h, double dt, int32_t nsteps, double *out_ms, int32_t cap) {
  if (!h || !out_ms || cap < 6 || nsteps <= 0) return hfail(h, SPC_ERR_INVALID, "bad argument");
  SPC_TRY(check_ready(h));
  return engine_profile(&h->e, dt, nsteps, out_ms);
}

int spc_set_tuning(spc_handle *h, int32_t key, double value) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  return engine_set_tuning(&h->e, key, value);
}

int spc_get_tuning(const spc_handle *h, int32_t key, double *value) {
  if (!h || !value) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  return engine_get_tuning(&h->e, key, value);
}

int spc_autotune(const spc_params *p, int32_t n, const double *aos3n, const double *omega, double dt,
                 int32_t trial_steps, spc_params *best, double *sparse_below, double *ms_out,
                 int32_t cap, int32_t *count) {
  if (!p || !aos3n || !best || !sparse_below || trial_steps <= 0)
    return fail(nullptr, SPC_ERR_INVALID, "bad argument");
  if (p->model == SPC_MODEL_VORTEX && !omega) return fail(nullptr, SPC_ERR_INVALID, "vortex model needs omega");
  std::string why;
  int rc = validate_params(p, n, why);
  if (rc) return fail(nullptr, rc, "%s", why.c_str());
  struct Cand {
    int neighbour;
    double skin, sparse;
  };
  std::vector<Cand> cands = {{SPC_NEIGHBOUR_CELL, p->skin, kSparseBelowDefault},
                             {SPC_NEIGHBOUR_CELL, p->skin, 0.0},
                             {SPC_NEIGHBOUR_CELL, p->skin, 1e9}};
  for (double f : {0.1, 0.2, 0.4}) {
    if (p->precision == SPC_PRECISION_FP32X) break;  // the FP32X form runs the cell list
    spc_params q = *p;
    q.neighbour = SPC_NEIGHBOUR_VERLET;
    q.skin = f * p->rho;
    if (make_sysconst(q, n).vR > 0) cands.push_back({SPC_NEIGHBOUR_VERLET, q.skin, kSparseBelowDefault});
  }
  double best_ms = 1e300;
  int best_k = -1;
  for (size_t k = 0; k < cands.size(); ++k) {
    spc_params q = *p;
    q.neighbour = cands[k].neighbour;
    q.skin = cands[k].skin;
    spc_handle *h = nullptr;
    rc = spc_create(&q, n, &h);
    if (rc == SPC_OK) rc = spc_upload_state(h, aos3n);
    if (rc == SPC_OK && omega) rc = spc_upload_omega(h, omega);
    if (rc == SPC_OK && cands[k].neighbour == SPC_NEIGHBOUR_CELL)
      rc = spc_set_tuning(h, SPC_TUNE_SPARSE_BELOW, cands[k].sparse);
    double t = 0.0, ms = 1e300;
    if (rc == SPC_OK) rc = spc_step_graph(h, &t, dt, trial_steps);  // capture + warm-up
    if (rc == SPC_OK) {
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      cudaError_t ce = cudaEventCreate(&e0);
      if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
      if (ce == cudaSuccess) ce = cudaEventRecord(e0, h->e.stream);
      if (ce == cudaSuccess) rc = spc_step_graph(h, &t, dt, trial_steps);
      if (ce == cudaSuccess && rc == SPC_OK) ce = cudaEventRecord(e1, h->e.stream);
      if (ce == cudaSuccess && rc == SPC_OK) ce = cudaEventSynchronize(e1);
      float f = 0.0f;
      if (ce == cudaSuccess && rc == SPC_OK) ce = cudaEventElapsedTime(&f, e0, e1);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      if (ce != cudaSuccess && rc == SPC_OK) rc = fail(nullptr, SPC_ERR_CUDA, "autotune timing: %s", cudaGetErrorString(ce));
      ms = (double)f / trial_steps;
    }
    std::string msg = h ? h->e.err : std::string();
    spc_destroy(h);
    if (rc != SPC_OK) return fail(nullptr, rc, "autotune candidate %d: %s", (int)k, msg.c_str());
    if (ms_out && (int)k < cap) ms_out[k] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best_k = (int)k;
    }
  }
  *best = *p;
  best->neighbour = cands[best_k].neighbour;
  best->skin = cands[best_k].skin;
  *sparse_below = cands[best_k].sparse;
  if (count) *count = (int32_t)cands.size();
  return SPC_OK;
}

int spc_autotune_ex(const spc_params *p, int32_t n, const double *aos3n, const double *omega, double dt,
                    int32_t trial_steps, spc_tuning *cands_out, int32_t cap, int32_t *count, int32_t *best) {
  if (!p || !aos3n || trial_steps <= 0) return fail(nullptr, SPC_ERR_INVALID, "bad argument");
  if (p->model == SPC_MODEL_VORTEX && !omega) return fail(nullptr, SPC_ERR_INVALID, "vortex model needs omega");
  std::string why;
  int rc = validate_params(p, n, why);
  if (rc) return fail(nullptr, rc, "%s", why.c_str());
  std::vector<spc_tuning> cands;
  for (const TuneCand &c : kernel_candidates(p->precision))
    cands.push_back({SPC_NEIGHBOUR_CELL, c.split, 0.0, c.sparse, 0.0, c.units, c.subcells});
  for (double f : {0.1, 0.2, 0.4}) {
    if (p->precision == SPC_PRECISION_FP32X) break;  // the FP32X form runs the cell list
    spc_params q = *p;
    q.neighbour = SPC_NEIGHBOUR_VERLET;
    q.skin = f * p->rho;
    if (make_sysconst(q, n).vR > 0)
      cands.push_back({SPC_NEIGHBOUR_VERLET, 1, q.skin, kSparseBelowDefault, 0.0, 0, 0});
  }
  int best_k = 0;
  for (size_t k = 0; k < cands.size(); ++k) {
    spc_params q = *p;
    q.neighbour = cands[k].neighbour;
    if (q.neighbour == SPC_NEIGHBOUR_VERLET) q.skin = cands[k].skin;
    spc_handle *h = nullptr;
    rc = spc_create(&q, n, &h);
    if (rc == SPC_OK) rc = spc_upload_state(h, aos3n);
    if (rc == SPC_OK && omega) rc = spc_upload_omega(h, omega);
    if (rc == SPC_OK && q.neighbour == SPC_NEIGHBOUR_CELL) {
      rc = spc_set_tuning(h, SPC_TUNE_SPARSE_BELOW, cands[k].sparse_below);
      if (rc == SPC_OK) rc = spc_set_tuning(h, SPC_TUNE_TILE_SPLIT, cands[k].tile_split);
      if (rc == SPC_OK) rc = spc_set_tuning(h, SPC_TUNE_CELL_UNITS, cands[k].cell_units);
      if (rc == SPC_OK) rc = spc_set_tuning(h, SPC_TUNE_SUBCELLS, cands[k].subcells);
    }
    double t = 0.0;
    float f = 0.0f;
    if (rc == SPC_OK) rc = spc_step_graph(h, &t, dt, trial_steps);  // capture + warm-up
    if (rc == SPC_OK) {
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      cudaError_t ce = cudaEventCreate(&e0);
      if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
      if (ce == cudaSuccess) ce = cudaEventRecord(e0, h->e.stream);
      if (ce == cudaSuccess) rc = spc_step_graph(h, &t, dt, trial_steps);
      if (ce == cudaSuccess && rc == SPC_OK) ce = cudaEventRecord(e1, h->e.stream);
      if (ce == cudaSuccess && rc == SPC_OK) ce = cudaEventSynchronize(e1);
      if (ce == cudaSuccess && rc == SPC_OK) ce = cudaEventElapsedTime(&f, e0, e1);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      if (ce != cudaSuccess && rc == SPC_OK)
        rc = fail(nullptr, SPC_ERR_CUDA, "autotune timing: %s", cudaGetErrorString(ce));
    }
    std::string msg = h ? h->e.err : std::string();
    spc_destroy(h);
    if (rc != SPC_OK) return fail(nullptr, rc, "autotune candidate %d: %s", (int)k, msg.c_str());
    cands[k].ms_per_step = (double)f / trial_steps;
    if (cands[k].ms_per_step < cands[best_k].ms_per_step) best_k = (int)k;
  }
  for (size_t k = 0; k < cands.size() && (int)k < cap && cands_out; ++k) cands_out[k] = cands[k];
  if (count) *count = (int32_t)cands.size();
  if (best) *best = best_k;
  return SPC_OK;
}

int spc_retune(spc_handle *h, double dt, int32_t trial_steps, spc_tuning *cands, int32_t cap, int32_t *count,
               int32_t *best) {
  if (!h) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(check_ready(h));
  int c = 0, b = 0;
  SPC_TRY(engine_retune(&h->e, dt, trial_steps, cands, cap, &c, &b));
  if (cands)
    for (int k = 0; k < std::min(c, (int)cap); ++k)
      cands[k].skin = h->p.neighbour == SPC_NEIGHBOUR_VERLET ? h->p.skin : 0.0;
  if (count) *count = c;
  if (best) *best = b;
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

int spc_check_division(int64_t n, const double *a, const double *b, int64_t *mismatches) {
  if (!a || !b || !mismatches || n < 0) return fail(nullptr, SPC_ERR_INVALID, "bad argument");
  *mismatches = 0;
  if (n == 0) return SPC_OK;
  double *da = nullptr, *db = nullptr;
  unsigned long long *dbad = nullptr;
  cudaError_t e = cudaMalloc(&da, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMalloc(&db, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dbad, 8);
  if (e == cudaSuccess) e = cudaMemcpy(da, a, (size_t)n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, b, (size_t)n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dbad, 0, 8);
  if (e == cudaSuccess) {
    k_check_division<<<152 * 8, 256>>>(n, da, db, dbad);
    e = cudaGetLastError();
  }
  unsigned long long bad = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&bad, dbad, 8, cudaMemcpyDeviceToHost);
  cudaFree(da);
  cudaFree(db);
  cudaFree(dbad);
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "check_division: %s", cudaGetErrorString(e));
  *mismatches = (int64_t)bad;
  return SPC_OK;
}

int spc_check_sincos(int64_t n, const double *x, int64_t *mismatches) {
  if (!x || !mismatches || n < 0) return fail(nullptr, SPC_ERR_INVALID, "bad argument");
  *mismatches = 0;
  if (n == 0) return SPC_OK;
  double *dx = nullptr, *ds = nullptr, *dc = nullptr;
  unsigned long long *dbad = nullptr;
  cudaError_t e = cudaMalloc(&dx, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMalloc(&ds, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dc, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dbad, 8);
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dbad, 0, 8);
  if (e == cudaSuccess) {
    k_sin_only<<<152 * 8, 256>>>(n, dx, ds);
    k_cos_only<<<152 * 8, 256>>>(n, dx, dc);
    k_sincos_cmp<<<152 * 8, 256>>>(n, dx, ds, dc, dbad);
    e = cudaGetLastError();
  }
  unsigned long long bad = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&bad, dbad, 8, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(ds);
  cudaFree(dc);
  cudaFree(dbad);
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "check_sincos: %s", cudaGetErrorString(e));
  *mismatches = (int64_t)bad;
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

// ===========================================================================
// Batches
int spc_batch_footprint(int32_t stepper, int32_t precision, int64_t *bytes_per_particle,
                        int64_t *bytes_per_cell) {
  long long bp = 0, bc = 0;
  engine_footprint(stepper, precision, &bp, &bc);
  if (bytes_per_particle) *bytes_per_particle = bp;
  if (bytes_per_cell) *bytes_per_cell = bc;
  return SPC_OK;
}

int spc_batch_create(const spc_batch_config *cfg, spc_batch **out) {
  if (!cfg || !out) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (cfg->max_systems <= 0 || cfg->max_particles <= 0 || cfg->max_cells <= 0 ||
      cfg->max_particles > (1ll << 30) || cfg->max_cells > (1ll << 30))
    return fail(nullptr, SPC_ERR_INVALID, "bad batch capacities");
  if (cfg->stepper < SPC_STEPPER_EULER || cfg->stepper > SPC_STEPPER_EULER_PTR)
    return fail(nullptr, SPC_ERR_INVALID, "unknown stepper");
  if (cfg->precision != SPC_PRECISION_FP64 && cfg->precision != SPC_PRECISION_FP32C &&
      cfg->precision != SPC_PRECISION_FP32X)
    return fail(nullptr, SPC_ERR_INVALID, "unknown precision");
  spc_batch *b = new spc_batch();
  int rc = engine_init(&b->e, cfg->stepper, cfg->precision, (int)cfg->max_particles, cfg->max_systems,
                       (int)cfg->max_cells);
  if (rc != SPC_OK) {
    std::string msg = b->e.err;
    engine_free(&b->e);
    delete b;
    fail(nullptr, rc, "%s", msg.c_str());
    return rc;
  }
  *out = b;
  return SPC_OK;
}

int spc_batch_destroy(spc_batch *b) {
  if (!b) return SPC_OK;
  engine_free(&b->e);
  delete b;
  return SPC_OK;
}

const char *spc_batch_last_error(const spc_batch *b) {
  if (b) return b->e.err.c_str();
  std::lock_guard<std::mutex> lk(err_mutex());
  return global_error().c_str();
}

int spc_batch_admit(spc_batch *b, const spc_params *p, int32_t n, const double *aos3n, const double *omega,
                    int64_t steps, int32_t *slot) {
  if (!b || !p || !aos3n || !slot) return fail(b ? &b->e : nullptr, SPC_ERR_INVALID, "NULL argument");
  Engine *e = &b->e;
  if (p->model == SPC_MODEL_VORTEX && !omega) return fail(e, SPC_ERR_INVALID, "vortex system needs omega");
  SPC_TRY(engine_set_device(e));
  int s = -1;
  SPC_TRY(engine_admit(e, *p, n, steps, &s));
  int rc = engine_upload(e, s, aos3n);
  if (rc == SPC_OK && omega) rc = engine_upload_omega(e, s, omega);
  if (rc == SPC_OK && e->stepper == SPC_STEPPER_RK4) {
    const SysHost &h = e->slots[s];
    for (int q = 0; q < 4 && rc == SPC_OK; ++q) {
      cudaError_t ce = cudaMemsetAsync(e->a.kx[q] + h.pool_p0, 0, (size_t)n * 8, e->stream);
      if (ce == cudaSuccess) ce = cudaMemsetAsync(e->a.ky[q] + h.pool_p0, 0, (size_t)n * 8, e->stream);
      if (ce == cudaSuccess) ce = cudaMemsetAsync(e->a.kphi[q] + h.pool_p0, 0, (size_t)n * 8, e->stream);
      if (ce != cudaSuccess) rc = fail(e, SPC_ERR_CUDA, "reset k: %s", cudaGetErrorString(ce));
    }
  }
  if (rc == SPC_OK) {
    cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) rc = fail(e, SPC_ERR_CUDA, "admit: %s", cudaGetErrorString(ce));
  }
  if (rc != SPC_OK) {
    engine_release(e, s);
    return rc;
  }
  *slot = s;
  return SPC_OK;
}

int spc_batch_release(spc_batch *b, int32_t slot) {
  if (!b) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  return engine_release(&b->e, slot);
}

int spc_batch_step(spc_batch *b, double dt, int32_t nsteps) {
  if (!b || nsteps < 0) return fail(b ? &b->e : nullptr, SPC_ERR_INVALID, "bad argument");
  return engine_steps(&b->e, dt, nsteps, false, nullptr, 0);
}

int spc_batch_step_graph(spc_batch *b, double dt, int32_t nsteps) {
  if (!b || nsteps <= 0) return fail(b ? &b->e : nullptr, SPC_ERR_INVALID, "bad argument");
  return engine_steps(&b->e, dt, nsteps, true, nullptr, 0);
}

int spc_batch_download(spc_batch *b, int32_t slot, double *aos3n) {
  if (!b || !aos3n) return fail(b ? &b->e : nullptr, SPC_ERR_INVALID, "NULL argument");
  if (!batch_slot_ok(b, slot)) return fail(&b->e, SPC_ERR_INVALID, "no system in slot %d", slot);
  SPC_TRY(engine_set_device(&b->e));
  return engine_download(&b->e, slot, aos3n);
}

int spc_batch_upload(spc_batch *b, int32_t slot, const double *aos3n) {
  if (!b || !aos3n) return fail(b ? &b->e : nullptr, SPC_ERR_INVALID, "NULL argument");
  if (!batch_slot_ok(b, slot)) return fail(&b->e, SPC_ERR_INVALID, "no system in slot %d", slot);
  SPC_TRY(engine_set_device(&b->e));
  SPC_TRY(engine_upload(&b->e, slot, aos3n));
  SPC_CUDA(&b->e, cudaStreamSynchronize(b->e.stream));
  return SPC_OK;
}

int spc_batch_status(spc_batch *b, int32_t slot, uint64_t *steps_done, int64_t *remaining) {
  if (!b) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  if (!batch_slot_ok(b, slot)) return fail(&b->e, SPC_ERR_INVALID, "no system in slot %d", slot);
  const SysHost &h = b->e.slots[slot];
  if (steps_done) *steps_done = h.step;
  if (remaining) *remaining = h.remaining;
  return SPC_OK;
}

int spc_batch_usage(spc_batch *b, int64_t *particles, int64_t *cells, int32_t *systems) {
  if (!b) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  long long used = 0;
  for (int s : b->e.order) used += b->e.slots[s].n;
  if (particles) *particles = used;
  if (cells) *cells = b->e.cells_used;
  if (systems) *systems = (int32_t)b->e.order.size();
  return SPC_OK;
}

int spc_batch_order_params(spc_batch *b, int32_t slot, double *R, double *psi) {
  if (!b) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  if (!batch_slot_ok(b, slot)) return fail(&b->e, SPC_ERR_INVALID, "no system in slot %d", slot);
  SPC_TRY(engine_set_device(&b->e));
  return engine_order_global(&b->e, slot, R, psi);
}

int spc_batch_order_params_all(spc_batch *b, int32_t cap, double *R, double *psi, double *R_local) {
  if (!b || cap < 0) return fail(b ? &b->e : nullptr, SPC_ERR_INVALID, "bad argument");
  SPC_TRY(engine_set_device(&b->e));
  return engine_order_all(&b->e, cap, R, psi, R_local);
}

int spc_batch_synchronize(spc_batch *b) {
  if (!b) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  SPC_TRY(engine_set_device(&b->e));
  SPC_CUDA(&b->e, cudaStreamSynchronize(b->e.stream));
  return SPC_OK;
}

void *spc_batch_stream(spc_batch *b) { return b ? (void *)b->e.stream : nullptr; }

int spc_batch_set_tuning(spc_batch *b, int32_t key, double value) {
  if (!b) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  return engine_set_tuning(&b->e, key, value);
}

int spc_batch_get_tuning(const spc_batch *b, int32_t key, double *value) {
  if (!b || !value) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  return engine_get_tuning(&b->e, key, value);
}

int spc_batch_retune(spc_batch *b, double dt, int32_t trial_steps, spc_tuning *cands, int32_t cap,
                     int32_t *count, int32_t *best) {
  if (!b) return fail(nullptr, SPC_ERR_INVALID, "NULL argument");
  int c = 0, k = 0;
  SPC_TRY(engine_retune(&b->e, dt, trial_steps, cands, cap, &c, &k));
  if (count) *count = c;
  if (best) *best = k;
  return SPC_OK;
}

int spc_batch_profile_steps(spc_batch *b, double dt, int32_t nsteps, double *out_ms, int32_t cap) {
  if (!b || !out_ms || cap < 6 || nsteps <= 0)
    return fail(b ? &b->e : nullptr, SPC_ERR_INVALID, "bad argument");
  return engine_profile(&b->e, dt, nsteps, out_ms);
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
// cell table, the cell-order copies, the one-entry system table) lives in one
// file-scope __device__ array of fixed size, resident on every GPU that loads
// this library until the process exits.
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
constexpr size_t kNaSys = na_round(sizeof(SysDesc));
// x y phi omega | st_x st_y st_phi | sx sy sphi | dphi_s      (11 double arrays)
// keys vals keys_alt vals_alt pidx cnt_s dphi_f sys_of_p      (8 32-bit arrays)
// fxy cs (2 float2 arrays) | cell_start | sys_of_c | hist | system table | all-pairs cell | clamp counter
constexpr size_t kNoAllocBytes =
    11 * kNaD + 8 * kNaF + 2 * kNaF2 + 2 * kNaCells + kNaHist + kNaSys + 256 + 256;

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
// per device: the array's device address and the unique ID of the context it
// was looked up in (a reset device gets a new context, and the module's
// arrays may then sit at other addresses)
char *g_noalloc_base[kNoAllocMaxDevices] = {};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

// Unique ID of the calling thread's current context, 0 when there is none
// or the driver does not report it.  The driver's cuCtxGetCurrent and
// cuCtxGetId are reached through the runtime's entry-point query, so the
// library does not link libcuda itself.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrent)(CUcontext *);
  typedef CUresult (*GetId)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
  });
  if (!get_current || !get_id) return 0;
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
  unsigned long long id = 0;
  return get_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

// Device address of g_noalloc_scratch on the current device.  In host code
// the symbol name is only a stand-in, so the address is looked up with the
// device current and cached per device together with the context it belongs
// to; a call in a different context (after cudaDeviceReset, say) looks it up
// again.  When the context's ID is unknown, every call looks it up.
int noalloc_scratch(char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(nullptr, SPC_ERR_INVALID, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_noalloc_base[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(nullptr, SPC_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_noalloc_base[dev] = (char *)ptr;
    // the lookup makes the device's primary context current if none was
    g_noalloc_ctx[dev] = current_context_id();
  }
  *out = g_noalloc_base[dev];
  return SPC_OK;
}

// Writes the one-entry system table (and the all-pairs cell) from kernel
// parameters, so no host-to-device copy is needed.
__global__ void k_noalloc_table(SysDesc *sys, SysDesc d, int *ap) {
  sys[0] = d;
  ap[0] = 0;
}

}  // namespace

extern "C" int spc_rhs_srk_noalloc(const spc_params *p, int32_t n, const double *d_state,
                                   double *d_derivative, double *d_additional, void *stream) {
  std::string why;
  int rc = validate_params(p, n, why);
  if (rc) return fail(nullptr, rc, "%s", why.c_str());
  if (!d_state || !d_derivative || !d_additional)
    return fail(nullptr, SPC_ERR_INVALID, "NULL device buffer");
  // the scratch holds the cell-list and all-pairs intermediates of the
  // alignment models; the vortex-arrays model's passes need tables of their own
  if (p->model == SPC_MODEL_VORTEX_ARRAYS)
    return fail(nullptr, SPC_ERR_INVALID,
                "spc_rhs_srk_noalloc: the vortex-arrays model is not supported (use spc_rhs_srk)");
  if (p->precision == SPC_PRECISION_FP32X)
    return fail(nullptr, SPC_ERR_INVALID,
                "spc_rhs_srk_noalloc: the FP32X form is not supported (FP64 and FP32C are)");
  if (n > kNoAllocMaxN)
    return fail(nullptr, SPC_ERR_CAPACITY, "spc_rhs_srk_noalloc: n = %d exceeds its maximum of %d particles",
                n, kNoAllocMaxN);
  const SysConst sc = make_sysconst(*p, n);
  const int ncell = sc.allpairs ? 1 : sc.ncell;
  if (ncell > kNoAllocMaxCells)
    return fail(nullptr, SPC_ERR_CAPACITY, "spc_rhs_srk_noalloc: %d x %d cells exceed its maximum of %d cells",
                sc.nc, sc.nc, kNoAllocMaxCells);
  char *base = nullptr;
  rc = noalloc_scratch(&base);
  if (rc) return rc;

  Engine e;  // a view: every device pointer below is inside the static scratch
  e.view = true;
  e.stepper = SPC_STEPPER_SRK;
  e.precision = p->precision;
  e.stream = (cudaStream_t)stream;
  KArgs &a = e.a;
  char *cur = base;
  auto take = [&](size_t bytes) {
    char *r = cur;
    cur += bytes;
    return (void *)r;
  };
  a.x = (double *)take(kNaD);
  a.y = (double *)take(kNaD);
  a.phi = (double *)take(kNaD);
  a.omega = (double *)take(kNaD);
  a.st_x = (double *)take(kNaD);
  a.st_y = (double *)take(kNaD);
  a.st_phi = (double *)take(kNaD);
  a.sx = (double *)take(kNaD);
  a.sy = (double *)take(kNaD);
  a.sphi = (double *)take(kNaD);
  a.dphi_s = (double *)take(kNaD);
  a.keys = (uint32_t *)take(kNaF);
  a.vals = (uint32_t *)take(kNaF);
  e.keys_alt = (uint32_t *)take(kNaF);
  e.vals_alt = (uint32_t *)take(kNaF);
  a.pidx = (int *)take(kNaF);
  a.cnt_s = (int *)take(kNaF);
  a.dphi_f = (float *)take(kNaF);
  int *sys_of_p = (int *)take(kNaF);
  a.fxy = (float2 *)take(kNaF2);
  a.cs = (float2 *)take(kNaF2);
  a.cell_start = (int *)take(kNaCells);
  int *sys_of_c = (int *)take(kNaCells);
  e.hist = (uint32_t *)take(kNaHist);
  SysDesc *sys = (SysDesc *)take(kNaSys);
  int *ap = (int *)take(256);
  unsigned long long *clamped = (unsigned long long *)take(256);
  a.sys_of_p = sys_of_p;
  a.sys_of_c = sys_of_c;
  a.sys = sys;
  a.ap_cells = ap;
  a.clamped = clamped;
  a.hist = e.hist;
  a.nbmask = nullptr;  // pass 2 re-tests candidates instead of reading masks
  a.out_d = d_derivative;
  a.out_a = d_additional;
  // layout of the single system
  e.nsys = 1;
  e.n_active = n;
  e.ncell_total = ncell;
  e.ntiles = (n + kSortTile - 1) / kSortTile;
  int bits = 1;
  while (bits < 31 && (1u << bits) < (unsigned)std::max(ncell, 2)) ++bits;
  e.sort_passes = (bits + 10) / 11;
  e.radix_bits = (bits + e.sort_passes - 1) / e.sort_passes;
  e.has_cells = !sc.allpairs;
  a.nsys = 1;
  a.n_active = n;
  a.ncell_total = ncell;
  a.ncell_tile = sc.allpairs ? 0 : ncell;  // cell-tile kernels only
  a.va_c0 = a.va_c1 = ncell;
  e.ncell_tile = a.ncell_tile;
  e.ncell_warp = 0;
  a.n_ap = sc.allpairs ? 1 : 0;
  e.ap_items = sc.allpairs ? (n + kAllPairsThreads - 1) / kAllPairsThreads : 0;
  e.ap_items_small = sc.allpairs ? (n + kAllPairsThreadsSmall - 1) / kAllPairsThreadsSmall : 0;
  a.hist_len = (1 << e.radix_bits) * e.ntiles;
  SysHost h;
  h.used = true;
  h.p = *p;
  h.n = n;
  h.pool_p0 = 0;
  h.ncell = ncell;
  h.sc = sc;
  const SysDesc d = desc_of(h, 0, 0);

  cudaError_t ce = set_kernel_attributes();
  if (ce != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "kernel attributes: %s", cudaGetErrorString(ce));
  // the scratch keeps the previous call's contents: the clamp counter and the
  // radix histogram table are accumulated into, and the system maps must read
  // system 0, so they are cleared here
  ce = cudaMemsetAsync(clamped, 0, 8, e.stream);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(e.hist, 0, (size_t)a.hist_len * 4, e.stream);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(sys_of_p, 0, (size_t)n * 4, e.stream);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(sys_of_c, 0, (size_t)ncell * 4, e.stream);
  if (ce != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "clear scratch: %s", cudaGetErrorString(ce));
  k_noalloc_table<<<1, 1, 0, e.stream>>>(sys, d, ap);
  k_aos_to_soa<<<blocks_for(n, 256), 256, 0, e.stream>>>(d_state, n, a.x, a.y, a.phi);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return fail(nullptr, SPC_ERR_CUDA, "launch: %s", cudaGetErrorString(ce));
  KArgs run = a;
  rc = eval_stage(&e, run, 0, -1, 0.0);
  if (rc == SPC_OK) rc = launch_pass(&e, run, kKindSin, kEpiSrk1);
  if (rc == SPC_OK) rc = launch_pass(&e, run, kKindCos2, kEpiSrk2Out);
  if (rc != SPC_OK) fail(nullptr, rc, "%s", e.err.c_str());
  return rc;
}
