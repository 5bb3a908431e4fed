// Drop-in C++ classes with the reference's names and signatures, forwarding
// the particle-update path to the GB300 library (include/spc_gb300.h).
//
// A program written against raven91/spc2_langevin_integration's
//   Thread, PeriodicBoundaryConditions, ChimeraSystem,
//   StochasticEulerStepper, StochasticRungeKuttaStepper, RungeKutta4Stepper
// compiles against this header instead of the reference's
// Parallelization/Thread.hpp, BoundaryConfiguration/PeriodicBoundaryConditions.hpp,
// DynamicalSystems/ChimeraSystem.hpp and Steppers/*.hpp, with its engine loop
// (SimulationEngine.cpp:149-161) unchanged.  VortexArraysSystem (an empty
// class in the reference, DynamicalSystems/VortexArraysSystem.hpp:8-11) is the
// alignment system with natural frequencies in the stochastic Runge-Kutta
// update (StochasticRungeKuttaStepperPtr.hpp:65).
//
// Semantics kept: DoStep advances the caller's std::vector state by one step
// (state on the device; the vector is uploaded when it differs from what the
// device holds and refreshed after the step), EvaluateRhs fills k_next /
// derivative / additional_derivative exactly as the reference does.  The
// device also applies the engine's wrap, so the engine's own
// ApplyPeriodicBoundaryConditions call afterwards is an identity.
// Errors raise std::runtime_error with the library's message (the reference
// has no error path; its UB cases become errors or counted clamps here).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <functional>
#include <vector>

#include "../../include/spc_gb300.h"

#ifndef SPC_DROPIN_NO_DEFINITIONS
// Definitions.hpp:17-22: the including program defines kN and kL.
typedef double Real;
const int kS = 3;
extern const int kN;
extern const Real kL;
#endif

// Parallelization/Thread.hpp:10-38: one rank owning every particle.
class Thread {
 public:
  Thread(int argc, char **argv);
  virtual ~Thread() = default;
  int GetRank() { return 0; }
  int GetNumberOfMpichThreads() { return 1; }
  int GetNumberOfParticlesPerMpichThread() { return kN; }
  const std::vector<int> &GetLoopIndices() const { return loop_indices_; }
  virtual bool IsRoot() const { return true; }
  virtual void SynchronizeVector(std::vector<Real> &) {}
  virtual void SynchronizeVectorThroughBuffer(std::vector<Real> &, std::vector<Real> &) {}
  virtual void BroadcastVector(std::vector<Real> &) {}
  virtual void SynchronizePrelinkedList(std::vector<int> &) const {}

 protected:
  std::vector<int> loop_indices_;
};

// BoundaryConfiguration/PeriodicBoundaryConditions.hpp:11-41 (class A distance
// and the wrap; host-side, same formulas).
class PeriodicBoundaryConditions {
 public:
  PeriodicBoundaryConditions(Thread *thread, Real x_size, Real y_size);
  void ClassAEffectiveParticleDistance(Real x_i, Real y_i, Real x_j, Real y_j, Real &dx, Real &dy);
  void ApplyPeriodicBoundaryConditions(Real x, Real y, Real &x_pbc, Real &y_pbc);
  void ApplyPeriodicBoundaryConditions(std::vector<Real> &system_state);
  void ApplyPeriodicBoundaryConditions(Real *const system_state, long size);
  Real GetXSize() const { return x_size_; }
  Real GetYSize() const { return y_size_; }

 private:
  Thread *thread_;
  Real x_size_, y_size_, x_rsize_, y_rsize_;
};

// Parallelization/ThreadSharedMemory.hpp:14-60: one rank on one shared-memory
// node; the shared windows of the reference live on the device here.
class ThreadSharedMemory : public Thread {
 public:
  ThreadSharedMemory(int argc, char **argv) : Thread(argc, argv) {}
  int GetRootRank() { return 0; }
  int GetSharedRootRank() { return 0; }
  bool IsSharedRoot() { return true; }
  using Thread::BroadcastVector;
  using Thread::SynchronizeVector;
  void SynchronizeVector(Real *const, long) {}
  void SynchronizeVectorThroughoutClusters(Real *const) {}
  void SynchronizeVectorThroughoutClusters(int *const) {}
  void BroadcastVector(Real *const, long) {}
};

// Shared machinery of the systems: one library handle per stepper kind,
// created on first use, plus the host/device coherence of the state vector.
class SpcSystemBase {
 public:
  SpcSystemBase(Thread *thread, int model, Real v_0, Real sigma, Real rho, Real alpha, Real D_phi,
                Real rho_0, PeriodicBoundaryConditions &pbc_config);
  virtual ~SpcSystemBase();
  SpcSystemBase(const SpcSystemBase &) = delete;
  SpcSystemBase &operator=(const SpcSystemBase &) = delete;

  Real rho() const { return rho_; }
  Real D_phi() const { return D_phi_; }
  Real alpha() const { return alpha_; }

  // GB300 extensions (no reference counterpart)
  void SetPrecision(int precision) { precision_ = precision; }
  void SetNeighbourSearch(int neighbour, Real skin) { neighbour_ = neighbour; skin_ = skin; }
  void SetSeed(uint64_t seed) { seed_ = seed; }
  // Feed these normals (reference draw order) to the next steps instead of Philox.
  void InjectNoise(const std::vector<Real> &normals) { injected_ = normals; inject_pending_ = true; }
  // nsteps steps of stepper kind `stepper` with one upload and one download.
  void Advance(int stepper, std::vector<Real> &state, Real &t, Real dt, int nsteps);
  // the same on a raw 3N state (the shared-window classes' Real * state)
  void AdvanceRaw(int stepper, Real *const state, Real &t, Real dt, int nsteps);
  // nsteps steps of the engine loop on the device (spc_run): after step k
  // (1-based) with observe[k % period] set, on_state(k, t_k, state) sees the
  // 3N state of that step while the device runs on; a true return stops the
  // run.  state and t end as after the steps taken, which are returned.
  using StateFn = std::function<bool(long, Real, const Real *)>;
  long Run(int stepper, std::vector<Real> &state, Real &t, Real dt, long nsteps, int period,
           const std::vector<uint8_t> &observe, const StateFn &on_state);
  // natural frequencies for the stochastic Runge-Kutta handle (re-uploaded
  // when they change)
  void UseFrequencies(const std::vector<Real> &frequencies);
  spc_handle *Handle(int stepper);

 protected:
  // the library model of the handle for stepper kind `stepper`
  virtual int ModelFor(int stepper) const { (void)stepper; return model_; }
  int SlotOf(const spc_handle *h) const;  // index of h in handles_
  void Sync(spc_handle *h, const std::vector<Real> &state);
  void Check(int rc, spc_handle *h) const;
  void RhsRk(const Real *state, const Real *k_prev, Real *k_next, Real k_coef, Real dt);
  void RhsSrk(const Real *state, Real *derivative, std::vector<std::vector<Real>> &additional);

  Thread *thread_;
  PeriodicBoundaryConditions &pbc_config_;
  int model_;
  Real v_0_, sigma_, rho_, alpha_, D_phi_, rho_0_;
  int precision_ = SPC_PRECISION_FP64;
  int neighbour_ = SPC_NEIGHBOUR_CELL;
  Real skin_ = 0.05;
  uint64_t seed_ = 0;
  std::vector<Real> frequencies_;
  bool omega_stale_[4] = {false, false, false, false};  // per handle: frequencies changed since its upload
  Real mu_plus_ = 0.0, mu_minus_ = 0.0, xi_a_ = 0.0, xi_r_ = 0.0, kappa_ = 0.0;  // vortex arrays
  spc_handle *handles_[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<Real> shadow_[4];  // what each handle's device state holds
  std::vector<Real> injected_;
  bool inject_pending_ = false;
};

// DynamicalSystems/ChimeraSystem.hpp:12-104
class ChimeraSystem : public SpcSystemBase {
 public:
  explicit ChimeraSystem(Thread *thread, Real v_0, Real sigma, Real rho, Real alpha, Real D_phi,
                         Real rho_0_, PeriodicBoundaryConditions &pbc_config);

  void EvaluateRhs(std::vector<Real> &system_state, const std::vector<Real> &k_prev,
                   std::vector<Real> &k_next, Real k_coef, Real dt);
  void EvaluateRhs(std::vector<Real> &system_state, std::vector<Real> &derivative,
                   std::vector<std::vector<Real>> &additional_derivative, Real dt);
  // stochastic part of the Euler method (ChimeraSystem.cpp:924-932), from the
  // same Philox stream the device steps use.
  void AddNoise(const std::vector<Real> &system_state, std::vector<Real> &derivative, Real t);

  bool should_accumulate_max_displacement_ = false;
};

// The vortex-array model: the alignment right-hand side with natural
// frequencies omega_i entering the SRK phase drift.
class VortexArraysSystem : public SpcSystemBase {
 public:
  VortexArraysSystem(Thread *thread, Real v_0, Real sigma, Real rho, Real D_phi, Real rho_0,
                     PeriodicBoundaryConditions &pbc_config, const std::vector<Real> &frequencies);
};

// DynamicalSystems/ChimeraSystemPtr.hpp:12-80: the alignment system of the
// shared-window classes.  With the stochastic Runge-Kutta stepper it takes the
// stepper's natural frequencies into the phase drift
// (StochasticRungeKuttaStepperPtr.hpp:65).
class ChimeraSystemPtr : public SpcSystemBase {
 public:
  ChimeraSystemPtr(ThreadSharedMemory *thread, Real v_0, Real sigma, Real rho, Real alpha, Real D_phi,
                   Real rho_0, PeriodicBoundaryConditions &pbc_config);
  void EvaluateRhs(const Real *const system_state, const std::vector<Real> &k_prev,
                   std::vector<Real> &k_next, Real k_coef, Real dt);
  void EvaluateRhs(const Real *const system_state, std::vector<Real> &derivative,
                   std::vector<std::vector<Real>> &additional_derivative, Real dt);
  bool last_coefficient_ = false;

 protected:
  int ModelFor(int stepper) const override {
    return stepper == SPC_STEPPER_SRK ? SPC_MODEL_VORTEX : SPC_MODEL_CHIMERA;
  }
};

// DynamicalSystems/VortexArraysSystemPtr.hpp:14-95: the vortex-arrays model.
class VortexArraysSystemPtr : public SpcSystemBase {
 public:
  VortexArraysSystemPtr(ThreadSharedMemory *thread, Real velocity, Real mu_plus, Real mu_minus,
                        Real xi_a, Real xi_r, Real D_phi, Real kappa, Real rho,
                        PeriodicBoundaryConditions &pbc_config);
  void EvaluateRhs(const Real *const system_state, const std::vector<Real> &k_prev,
                   std::vector<Real> &k_next, Real k_coef, Real dt);
  void EvaluateRhs(const Real *const system_state, std::vector<Real> &derivative,
                   std::vector<std::vector<Real>> &additional_derivative, Real dt);
  bool last_coefficient_ = false;
};

// Steppers/StochasticEulerStepper.hpp:15-47
class StochasticEulerStepper {
 public:
  explicit StochasticEulerStepper(Thread *thread) : thread_(thread) {}
  void DoStep(ChimeraSystem &chimera_system, std::vector<Real> &x, Real t, Real dt);

 private:
  Thread *thread_;
};

// Steppers/StochasticRungeKuttaStepper.hpp:15-61 (and the frequency form of
// StochasticRungeKuttaStepperPtr.hpp:41-68 for VortexArraysSystem)
class StochasticRungeKuttaStepper {
 public:
  explicit StochasticRungeKuttaStepper(Thread *thread) : thread_(thread) {}
  void DoStep(ChimeraSystem &system, std::vector<Real> &system_state, Real t, Real dt);
  void DoStep(VortexArraysSystem &system, std::vector<Real> &system_state, Real t, Real dt);

 private:
  Thread *thread_;
};

// Steppers/RungeKutta4Stepper.hpp:10-26 (k buffers persist on the device)
class RungeKutta4Stepper {
 public:
  explicit RungeKutta4Stepper(Thread *thread) : thread_(thread) {}
  void DoStep(ChimeraSystem &chimera_system, std::vector<Real> &system_state, Real t, Real dt);

 private:
  Thread *thread_;
};

// Steppers/StochasticEulerStepperPtr.hpp:14-80
class StochasticEulerStepperPtr {
 public:
  explicit StochasticEulerStepperPtr(ThreadSharedMemory *thread) : thread_(thread) {}
  void DoStep(ChimeraSystemPtr &system, Real *const system_state, Real t, Real dt);
  void DoStep(VortexArraysSystemPtr &system, Real *const system_state, Real t, Real dt);

 private:
  ThreadSharedMemory *thread_;
};

// Steppers/StochasticRungeKuttaStepperPtr.hpp:21-100.  The reference's
// constructor draws the natural frequencies from N(0, 0), i.e. all zero
// (:29-34); SetFrequencies (no reference counterpart) gives other ones.
class StochasticRungeKuttaStepperPtr {
 public:
  explicit StochasticRungeKuttaStepperPtr(ThreadSharedMemory *thread)
      : thread_(thread), frequencies_((size_t)kN, 0.0) {}
  void SetFrequencies(const std::vector<Real> &frequencies);
  void DoStep(ChimeraSystemPtr &system, Real *const system_state, Real t, Real dt);
  void DoStep(VortexArraysSystemPtr &system, Real *const system_state, Real t, Real dt);

 private:
  ThreadSharedMemory *thread_;
  std::vector<Real> frequencies_;
};

// Steppers/RungeKutta4StepperPtr.hpp:14-33 (k buffers persist on the device)
class RungeKutta4StepperPtr {
 public:
  explicit RungeKutta4StepperPtr(ThreadSharedMemory *thread) : thread_(thread) {}
  void DoStep(ChimeraSystemPtr &system, Real *const system_state, Real t, Real dt);
  void DoStep(VortexArraysSystemPtr &system, Real *const system_state, Real t, Real dt);

 private:
  ThreadSharedMemory *thread_;
};
