// Drop-in classes (spc_dropin.hpp) forwarding to the C-ABI.
#include "spc_dropin.hpp"

#include <algorithm>
#include <exception>
#include <cmath>
#include <numeric>

Thread::Thread(int, char **) : loop_indices_(kN) {
  std::iota(loop_indices_.begin(), loop_indices_.end(), 0);
}

PeriodicBoundaryConditions::PeriodicBoundaryConditions(Thread *thread, Real x_size, Real y_size)
    : thread_(thread), x_size_(x_size), y_size_(y_size), x_rsize_(1.0 / x_size),
      y_rsize_(1.0 / y_size) {}

void PeriodicBoundaryConditions::ClassAEffectiveParticleDistance(Real x_i, Real y_i, Real x_j,
                                                                 Real y_j, Real &dx, Real &dy) {
  dx = x_j - x_i;
  dx -= static_cast<int>(dx * 2.0 * x_rsize_) * x_size_;
  dy = y_j - y_i;
  dy -= static_cast<int>(dy * 2.0 * y_rsize_) * y_size_;
}

void PeriodicBoundaryConditions::ApplyPeriodicBoundaryConditions(Real x, Real y, Real &x_pbc,
                                                                 Real &y_pbc) {
  x_pbc = x - std::floor(x * x_rsize_) * x_size_;
  y_pbc = y - std::floor(y * y_rsize_) * y_size_;
}

void PeriodicBoundaryConditions::ApplyPeriodicBoundaryConditions(std::vector<Real> &s) {
  ApplyPeriodicBoundaryConditions(s.data(), (long)s.size());
}

void PeriodicBoundaryConditions::ApplyPeriodicBoundaryConditions(Real *const s, long size) {
  // The device already wrapped the state it returned, and the wrap is
  // idempotent on [0, L), so this leaves a device-produced state unchanged.
  for (long ii = 0; ii + 1 < size; ii += kS) {
    s[ii] -= std::floor(s[ii] * x_rsize_) * x_size_;
    s[ii + 1] -= std::floor(s[ii + 1] * y_rsize_) * y_size_;
  }
}

// ---------------------------------------------------------------------------
SpcSystemBase::SpcSystemBase(Thread *thread, int model, Real v_0, Real sigma, Real rho, Real alpha,
                             Real D_phi, Real rho_0, PeriodicBoundaryConditions &pbc_config)
    : thread_(thread), pbc_config_(pbc_config), model_(model), v_0_(v_0), sigma_(sigma),
      rho_(rho), alpha_(alpha), D_phi_(D_phi), rho_0_(rho_0) {}

SpcSystemBase::~SpcSystemBase() {
  for (spc_handle *&h : handles_) {
    spc_destroy(h);
    h = nullptr;
  }
}

void SpcSystemBase::Check(int rc, spc_handle *h) const {
  if (rc != SPC_OK) throw std::runtime_error(std::string("spc: ") + spc_last_error(h));
}

spc_handle *SpcSystemBase::Handle(int stepper) {
  if (!handles_[stepper]) {
    spc_params p{};
    p.model = ModelFor(stepper);
    p.stepper = stepper;
    p.neighbour = neighbour_;
    p.precision = precision_;
    p.L = pbc_config_.GetXSize();
    p.v0 = v_0_;
    p.sigma = sigma_;
    p.rho = rho_;
    p.alpha = alpha_;
    p.D_phi = D_phi_;
    p.rho_0 = rho_0_;
    p.skin = skin_;
    p.seed = seed_;
    p.mu_plus = mu_plus_;
    p.mu_minus = mu_minus_;
    p.xi_a = xi_a_;
    p.xi_r = xi_r_;
    p.kappa = kappa_;
    spc_handle *h = nullptr;
    Check(spc_create(&p, kN, &h), nullptr);
    handles_[stepper] = h;
    if (p.model == SPC_MODEL_VORTEX) {
      if ((int)frequencies_.size() != kN) frequencies_.assign((size_t)kN, 0.0);
      Check(spc_upload_omega(h, frequencies_.data()), h);
    }
    omega_stale_[stepper] = false;
  } else if (omega_stale_[stepper] && ModelFor(stepper) == SPC_MODEL_VORTEX) {
    Check(spc_upload_omega(handles_[stepper], frequencies_.data()), handles_[stepper]);
    omega_stale_[stepper] = false;
  }
  return handles_[stepper];
}

void SpcSystemBase::UseFrequencies(const std::vector<Real> &frequencies) {
  if ((int)frequencies.size() != kN) throw std::runtime_error("spc: need N frequencies");
  if (frequencies != frequencies_) {
    frequencies_ = frequencies;
    for (bool &stale : omega_stale_) stale = true;  // every handle uploads them on its next use
  }
}

void SpcSystemBase::AdvanceRaw(int stepper, Real *const state, Real &t, Real dt, int nsteps) {
  std::vector<Real> v(state, state + (size_t)kS * kN);
  Advance(stepper, v, t, dt, nsteps);
  std::copy(v.begin(), v.end(), state);
}

void SpcSystemBase::RhsRk(const Real *state, const Real *k_prev, Real *k_next, Real k_coef, Real dt) {
  spc_handle *h = Handle(SPC_STEPPER_RK4);
  Sync(h, std::vector<Real>(state, state + (size_t)kS * kN));
  Check(spc_rhs_rk(h, k_prev, k_coef, dt, k_next), h);
}

void SpcSystemBase::RhsSrk(const Real *state, Real *derivative,
                           std::vector<std::vector<Real>> &additional_derivative) {
  spc_handle *h = Handle(SPC_STEPPER_RK4);
  Sync(h, std::vector<Real>(state, state + (size_t)kS * kN));
  std::vector<Real> d(kS * (size_t)kN), a(2 * (size_t)kN);
  Check(spc_rhs_srk(h, d.data(), a.data()), h);
  // the steppers pass zero-filled buffers (StochasticRungeKuttaStepper.hpp:36-39)
  for (int i = 0; i < kN; ++i) {
    derivative[kS * i] = d[kS * i];
    derivative[kS * i + 1] = d[kS * i + 1];
    derivative[kS * i + 2] += d[kS * i + 2];
    additional_derivative[i][0] += a[2 * i];
    additional_derivative[i][1] += a[2 * i + 1];
  }
}

int SpcSystemBase::SlotOf(const spc_handle *h) const {
  int k = 0;
  while (handles_[k] != h) ++k;
  return k;
}

void SpcSystemBase::Sync(spc_handle *h, const std::vector<Real> &state) {
  const int k = SlotOf(h);
  if (shadow_[k] != state) {
    Check(spc_upload_state(h, state.data()), h);
    shadow_[k] = state;
  }
}

void SpcSystemBase::Advance(int stepper, std::vector<Real> &state, Real &t, Real dt, int nsteps) {
  if ((int)state.size() != kS * kN) throw std::runtime_error("spc: state size is not 3N");
  spc_handle *h = Handle(stepper);
  Sync(h, state);
  if (inject_pending_) {
    Check(spc_inject_noise(h, injected_.data(), (int64_t)injected_.size()), h);
    inject_pending_ = false;
  }
  // the device state moves from here on: until the new state is back on the
  // host, no shadow claims to know it (a failed call re-uploads next time)
  const int k = SlotOf(h);
  shadow_[k].clear();
  double tt = t;
  Check(spc_step(h, &tt, dt, nsteps), h);
  Check(spc_download_state(h, state.data()), h);
  shadow_[k] = state;
  t = tt;
}

namespace {
struct RunCall {
  const SpcSystemBase::StateFn *fn;
  std::exception_ptr error;
};

int run_trampoline(void *user, int64_t step, double t, const double *aos3n) {
  RunCall *c = static_cast<RunCall *>(user);
  try {
    return (*c->fn)((long)step, t, aos3n) ? 1 : 0;
  } catch (...) {  // never unwind through the C library
    c->error = std::current_exception();
    return 1;
  }
}
}  // namespace

long SpcSystemBase::Run(int stepper, std::vector<Real> &state, Real &t, Real dt, long nsteps, int period,
                        const std::vector<uint8_t> &observe, const StateFn &on_state) {
  if ((int)state.size() != kS * kN) throw std::runtime_error("spc: state size is not 3N");
  if (on_state && (int)observe.size() != period) throw std::runtime_error("spc: observe needs period entries");
  spc_handle *h = Handle(stepper);
  Sync(h, state);
  if (inject_pending_) {
    Check(spc_inject_noise(h, injected_.data(), (int64_t)injected_.size()), h);
    inject_pending_ = false;
  }
  const int k = SlotOf(h);
  shadow_[k].clear();  // as in Advance: an error or a throwing observer re-uploads next time
  RunCall call{&on_state, nullptr};
  double tt = t;
  int64_t done = 0;
  const int rc = spc_run(h, &tt, dt, nsteps, period, on_state ? observe.data() : nullptr,
                         on_state ? run_trampoline : nullptr, &call, &done);
  if (call.error) std::rethrow_exception(call.error);
  Check(rc, h);
  Check(spc_download_state(h, state.data()), h);
  shadow_[k] = state;
  t = tt;
  return (long)done;
}

// ---------------------------------------------------------------------------
ChimeraSystem::ChimeraSystem(Thread *thread, Real v_0, Real sigma, Real rho, Real alpha,
                             Real D_phi, Real rho_0, PeriodicBoundaryConditions &pbc_config)
    : SpcSystemBase(thread, SPC_MODEL_CHIMERA, v_0, sigma, rho, alpha, D_phi, rho_0, pbc_config) {}

void ChimeraSystem::EvaluateRhs(std::vector<Real> &system_state, const std::vector<Real> &k_prev,
                                std::vector<Real> &k_next, Real k_coef, Real dt) {
  RhsRk(system_state.data(), k_prev.data(), k_next.data(), k_coef, dt);
}

void ChimeraSystem::EvaluateRhs(std::vector<Real> &system_state, std::vector<Real> &derivative,
                                std::vector<std::vector<Real>> &additional_derivative, Real dt) {
  (void)dt;
  RhsSrk(system_state.data(), derivative.data(), additional_derivative);
}

void ChimeraSystem::AddNoise(const std::vector<Real> &, std::vector<Real> &derivative, Real) {
  spc_handle *h = Handle(SPC_STEPPER_EULER);
  uint64_t step = 0;
  Check(spc_get_step_counter(h, &step), h);
  std::vector<Real> xi((size_t)kN);
  Check(spc_export_noise(h, step, 1, xi.data()), h);
  const Real intensity = std::sqrt(2.0 * D_phi_);
  for (int i = 0; i < kN; ++i) derivative[kS * i + 2] = intensity * xi[i];
}

VortexArraysSystem::VortexArraysSystem(Thread *thread, Real v_0, Real sigma, Real rho, Real D_phi,
                                       Real rho_0, PeriodicBoundaryConditions &pbc_config,
                                       const std::vector<Real> &frequencies)
    : SpcSystemBase(thread, SPC_MODEL_VORTEX, v_0, sigma, rho, 0.0, D_phi, rho_0, pbc_config) {
  frequencies_ = frequencies;
  if ((int)frequencies_.size() != kN) throw std::runtime_error("spc: need N frequencies");
}

void StochasticEulerStepper::DoStep(ChimeraSystem &chimera_system, std::vector<Real> &x, Real t,
                                    Real dt) {
  chimera_system.Advance(SPC_STEPPER_EULER, x, t, dt, 1);
}

void StochasticRungeKuttaStepper::DoStep(ChimeraSystem &system, std::vector<Real> &system_state,
                                         Real t, Real dt) {
  system.Advance(SPC_STEPPER_SRK, system_state, t, dt, 1);
}

void StochasticRungeKuttaStepper::DoStep(VortexArraysSystem &system,
                                         std::vector<Real> &system_state, Real t, Real dt) {
  system.Advance(SPC_STEPPER_SRK, system_state, t, dt, 1);
}

void RungeKutta4Stepper::DoStep(ChimeraSystem &chimera_system, std::vector<Real> &system_state,
                                Real t, Real dt) {
  chimera_system.Advance(SPC_STEPPER_RK4, system_state, t, dt, 1);
}

// ---------------------------------------------------------------------------
// shared-window classes
ChimeraSystemPtr::ChimeraSystemPtr(ThreadSharedMemory *thread, Real v_0, Real sigma, Real rho, Real alpha,
                                   Real D_phi, Real rho_0, PeriodicBoundaryConditions &pbc_config)
    : SpcSystemBase(thread, SPC_MODEL_CHIMERA, v_0, sigma, rho, alpha, D_phi, rho_0, pbc_config) {}

void ChimeraSystemPtr::EvaluateRhs(const Real *const system_state, const std::vector<Real> &k_prev,
                                   std::vector<Real> &k_next, Real k_coef, Real dt) {
  RhsRk(system_state, k_prev.data(), k_next.data(), k_coef, dt);
}

void ChimeraSystemPtr::EvaluateRhs(const Real *const system_state, std::vector<Real> &derivative,
                                   std::vector<std::vector<Real>> &additional_derivative, Real) {
  RhsSrk(system_state, derivative.data(), additional_derivative);
}

VortexArraysSystemPtr::VortexArraysSystemPtr(ThreadSharedMemory *thread, Real velocity, Real mu_plus,
                                             Real mu_minus, Real xi_a, Real xi_r, Real D_phi, Real kappa,
                                             Real rho, PeriodicBoundaryConditions &pbc_config)
    : SpcSystemBase(thread, SPC_MODEL_VORTEX_ARRAYS, velocity, 0.0, rho, 0.0, D_phi, 1.0, pbc_config) {
  mu_plus_ = mu_plus;
  mu_minus_ = mu_minus;
  xi_a_ = xi_a;
  xi_r_ = xi_r;
  kappa_ = kappa;
}

void VortexArraysSystemPtr::EvaluateRhs(const Real *const system_state, const std::vector<Real> &k_prev,
                                        std::vector<Real> &k_next, Real k_coef, Real dt) {
  RhsRk(system_state, k_prev.data(), k_next.data(), k_coef, dt);
}

void VortexArraysSystemPtr::EvaluateRhs(const Real *const system_state, std::vector<Real> &derivative,
                                        std::vector<std::vector<Real>> &additional_derivative, Real) {
  RhsSrk(system_state, derivative.data(), additional_derivative);
}

void StochasticEulerStepperPtr::DoStep(ChimeraSystemPtr &system, Real *const system_state, Real t, Real dt) {
  system.AdvanceRaw(SPC_STEPPER_EULER_PTR, system_state, t, dt, 1);
}

void StochasticEulerStepperPtr::DoStep(VortexArraysSystemPtr &system, Real *const system_state, Real t,
                                       Real dt) {
  system.AdvanceRaw(SPC_STEPPER_EULER_PTR, system_state, t, dt, 1);
}

void StochasticRungeKuttaStepperPtr::SetFrequencies(const std::vector<Real> &frequencies) {
  if ((int)frequencies.size() != kN) throw std::runtime_error("spc: need N frequencies");
  frequencies_ = frequencies;
}

void StochasticRungeKuttaStepperPtr::DoStep(ChimeraSystemPtr &system, Real *const system_state, Real t,
                                            Real dt) {
  system.UseFrequencies(frequencies_);
  system.AdvanceRaw(SPC_STEPPER_SRK, system_state, t, dt, 1);
}

void StochasticRungeKuttaStepperPtr::DoStep(VortexArraysSystemPtr &system, Real *const system_state, Real t,
                                            Real dt) {
  system.AdvanceRaw(SPC_STEPPER_SRK, system_state, t, dt, 1);
}

void RungeKutta4StepperPtr::DoStep(ChimeraSystemPtr &system, Real *const system_state, Real t, Real dt) {
  system.AdvanceRaw(SPC_STEPPER_RK4, system_state, t, dt, 1);
}

void RungeKutta4StepperPtr::DoStep(VortexArraysSystemPtr &system, Real *const system_state, Real t,
                                   Real dt) {
  system.AdvanceRaw(SPC_STEPPER_RK4, system_state, t, dt, 1);
}
