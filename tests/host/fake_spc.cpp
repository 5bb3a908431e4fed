// A host-memory stand-in for the C-ABI calls the drop-in adapters make
// (include/spc_gb300.h), for testing the adapters' own logic on a machine
// without a GPU: which state and frequencies reach which handle, and what
// happens after a failed call.
//
// Its "device" step is deliberately simple: every step moves each phase by
// dt * omega_i for a VORTEX-model handle and by dt for a CHIMERA-model one, and
// leaves positions alone, so a test can read from the final phases which
// frequencies a handle stepped with and from which state it started.
#include <cstring>
#include <vector>

#include "../../include/spc_gb300.h"

struct spc_handle {
  spc_params p;
  int n;
  std::vector<double> state, omega;
  uint64_t step = 0;
  long state_uploads = 0, omega_uploads = 0;
};

namespace {
int g_fail_after = -1;  // >= 0: the next spc_step / spc_run takes that many steps, then fails

void one_step(spc_handle *h, double dt) {
  for (int i = 0; i < h->n; ++i)
    h->state[3 * (size_t)i + 2] += dt * (h->p.model == SPC_MODEL_VORTEX ? h->omega[i] : 1.0);
  ++h->step;
}
}  // namespace

extern "C" {

// test controls (not part of the library's interface)
void fake_spc_fail_next_step(int after_steps) { g_fail_after = after_steps; }
long fake_spc_state_uploads(const spc_handle *h) { return h->state_uploads; }
long fake_spc_omega_uploads(const spc_handle *h) { return h->omega_uploads; }

const char *spc_last_error(const spc_handle *) { return "fake failure"; }

int spc_create(const spc_params *p, int32_t n, spc_handle **out) {
  spc_handle *h = new spc_handle();
  h->p = *p;
  h->n = n;
  h->state.assign(3 * (size_t)n, 0.0);
  h->omega.assign((size_t)n, 0.0);
  *out = h;
  return SPC_OK;
}

int spc_destroy(spc_handle *h) {
  delete h;
  return SPC_OK;
}

int spc_upload_state(spc_handle *h, const double *aos3n) {
  std::memcpy(h->state.data(), aos3n, h->state.size() * sizeof(double));
  ++h->state_uploads;
  return SPC_OK;
}

int spc_download_state(spc_handle *h, double *aos3n) {
  std::memcpy(aos3n, h->state.data(), h->state.size() * sizeof(double));
  return SPC_OK;
}

int spc_upload_omega(spc_handle *h, const double *omega) {
  std::memcpy(h->omega.data(), omega, h->omega.size() * sizeof(double));
  ++h->omega_uploads;
  return SPC_OK;
}

int spc_step(spc_handle *h, double *t_inout, double dt, int32_t nsteps) {
  for (int k = 0; k < nsteps; ++k) {
    if (g_fail_after == k) {
      g_fail_after = -1;
      return SPC_ERR_CUDA;
    }
    one_step(h, dt);
    *t_inout += dt;
  }
  return SPC_OK;
}

int spc_run(spc_handle *h, double *t_inout, double dt, int64_t nsteps, int32_t period,
            const uint8_t *observe, spc_observe_fn fn, void *user, int64_t *steps_done) {
  int64_t k = 0;
  while (k < nsteps) {
    if (g_fail_after == k) {
      g_fail_after = -1;
      *steps_done = k;
      return SPC_ERR_CUDA;
    }
    one_step(h, dt);
    *t_inout += dt;
    ++k;
    if (fn && observe && observe[k % period] && fn(user, k, *t_inout, h->state.data())) break;
  }
  *steps_done = k;
  return SPC_OK;
}

int spc_get_step_counter(const spc_handle *h, uint64_t *out) {
  *out = h->step;
  return SPC_OK;
}

int spc_inject_noise(spc_handle *, const double *, int64_t) { return SPC_OK; }

int spc_export_noise(spc_handle *h, uint64_t, int32_t nsteps, double *out) {
  std::memset(out, 0, (size_t)nsteps * h->n * sizeof(double));
  return SPC_OK;
}

int spc_rhs_rk(spc_handle *h, const double *, double, double, double *k_next) {
  std::memset(k_next, 0, h->state.size() * sizeof(double));
  return SPC_OK;
}

int spc_rhs_srk(spc_handle *h, double *derivative, double *additional) {
  std::memset(derivative, 0, h->state.size() * sizeof(double));
  std::memset(additional, 0, 2 * (size_t)h->n * sizeof(double));
  return SPC_OK;
}

}  // extern "C"
