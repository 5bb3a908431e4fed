// The reference's engine loop (SimulationEngine.cpp:149-161) written against
// the drop-in classes of spc_dropin.hpp, reading the same input format as the
// oracle's reference driver, so a test can show that a reference-style C++
// caller gets the reference's trajectory from the GPU path.
//
// usage: SPC_REF_N=<N> SPC_REF_L=<L> spc_dropin_driver <input.bin> <output.bin>
// (mode 0 = run the engine loop, modes 1/2 = one EvaluateRhs of either form,
//  mode 3 = the engine loop of SimulationEngine.cpp:113-127 for the vector
//  classes: the observer's frame at t0, then a frame and a summary line after
//  every step, and every state written to the output;
//  family 0 = vector classes, family 1 = shared-window classes, whose SRK
//  stepper takes the first N injected values as its natural frequencies,
//  family 2 = VortexArraysSystemPtr with the shared-window steppers, whose
//  five extra parameters follow the noise block and whose SRK stepper skips
//  the first N injected values, the frequencies it draws and never uses.)
// With SPC_OUTPUT_DIR set, a run also writes the reference's observer files
// there (a frame and a summary line after every step, as the engine loop does).
// With SPC_DEVICE_LOOP=1 a run is one RunObserved call (the loop on the
// device, states delivered at the observer's and the recording cadence)
// instead of one DoStep per step; the outputs must not change.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "spc_dropin.hpp"
#include "spc_observer.hpp"

static int env_int(const char *k) {
  const char *v = std::getenv(k);
  if (!v) std::exit(2);
  return std::atoi(v);
}
static double env_double(const char *k) {
  const char *v = std::getenv(k);
  if (!v) std::exit(2);
  return std::strtod(v, nullptr);
}
extern const int kN = env_int("SPC_REF_N");
extern const Real kL = env_double("SPC_REF_L");

struct Header {
  char magic[8];
  int32_t mode, family, stepper, nsteps, record_every, pad;
  double v0, sigma, rho, alpha, D_phi, rho_0, t0, dt, k_coef;
};

static void read_exact(FILE *f, void *p, size_t n) {
  if (std::fread(p, 1, n, f) != n) std::exit(2);
}

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  Header h;
  read_exact(in, &h, sizeof(h));
  if (std::memcmp(h.magic, "SPCREF01", 8) != 0) return 2;
  const size_t n3 = (size_t)kS * kN;
  std::vector<Real> state(n3), k_prev(n3), k_next(n3);
  read_exact(in, state.data(), n3 * 8);
  read_exact(in, k_prev.data(), n3 * 8);
  read_exact(in, k_next.data(), n3 * 8);
  int64_t n_noise = 0;
  read_exact(in, &n_noise, 8);
  std::vector<Real> noise((size_t)n_noise);
  if (n_noise) read_exact(in, noise.data(), (size_t)n_noise * 8);
  double va[5] = {0, 0, 0, 0, 0};  // mu_plus, mu_minus, xi_a, xi_r, kappa
  if (h.family == 2) read_exact(in, va, sizeof(va));
  std::fclose(in);
  FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  auto dump = [&](const Real *p, size_t n) { std::fwrite(p, 8, n, out); };
  try {
    ThreadSharedMemory thread(argc, argv);  // a Thread for the vector classes
    PeriodicBoundaryConditions pbc_config(&thread, kL, kL);
    BinaryObserver *observer = nullptr;
    if (std::getenv("SPC_OUTPUT_DIR") && (h.mode == 0 || h.mode == 3))
      observer = new BinaryObserver(&thread, h.v0, h.sigma, h.rho, h.alpha, h.D_phi, h.rho_0, pbc_config,
                                    h.dt, 0);
    auto observe = [&](std::vector<Real> &s, Real t) {
      if (!observer) return;
      observer->SaveSystemState(s, t);
      observer->SaveSummaryStatistics(s, t);
    };
    const bool device_loop = std::getenv("SPC_DEVICE_LOOP") && std::atoi(std::getenv("SPC_DEVICE_LOOP")) != 0;
    // the whole loop in one call: records every record_every-th state and the last
    auto run_device = [&](SpcSystemBase &system, int kind) {
      Real t = h.t0;
      RunObserved(system, kind, state, t, h.dt, h.nsteps, observer, h.record_every,
                  [&](long, Real, const std::vector<Real> &s) { dump(s.data(), n3); });
      if (h.record_every <= 0 || h.nsteps % h.record_every != 0) dump(state.data(), n3);
    };
    // the shared-window engine loop (SimulationEnginePtr.cpp:106-115)
    auto run_ptr = [&](auto &system) {
      if (h.mode == 1) {
        system.EvaluateRhs(state.data(), k_prev, k_next, h.k_coef, h.dt);
        dump(k_next.data(), n3);
        return;
      }
      if (h.mode == 2) {
        std::vector<Real> derivative(n3, 0.0);
        std::vector<std::vector<Real>> additional(kN, std::vector<Real>(2, 0.0));
        system.EvaluateRhs(state.data(), derivative, additional, h.dt);
        dump(derivative.data(), n3);
        for (int i = 0; i < kN; ++i) dump(additional[i].data(), 2);
        return;
      }
      StochasticEulerStepperPtr euler(&thread);
      StochasticRungeKuttaStepperPtr srk(&thread);
      RungeKutta4StepperPtr rk4(&thread);
      std::vector<Real> rest = noise;
      if (h.stepper == 1) {
        if ((int)noise.size() < kN) throw std::runtime_error("spc: SRK needs N frequencies first");
        if (h.family == 1) srk.SetFrequencies(std::vector<Real>(noise.begin(), noise.begin() + kN));
        rest.assign(noise.begin() + kN, noise.end());
      }
      if (!rest.empty()) system.InjectNoise(rest);
      if (device_loop) {
        if (h.stepper == 1 && h.family == 1)
          system.UseFrequencies(std::vector<Real>(noise.begin(), noise.begin() + kN));
        run_device(system, h.stepper == 0 ? SPC_STEPPER_EULER_PTR : h.stepper == 1 ? SPC_STEPPER_SRK : SPC_STEPPER_RK4);
        return;
      }
      Real t = h.t0;
      for (int k = 1; k <= h.nsteps; ++k) {
        t += h.dt;
        if (h.stepper == 0)
          euler.DoStep(system, state.data(), t, h.dt);
        else if (h.stepper == 1)
          srk.DoStep(system, state.data(), t, h.dt);
        else
          rk4.DoStep(system, state.data(), t, h.dt);
        pbc_config.ApplyPeriodicBoundaryConditions(state);
        thread.SynchronizeVectorThroughoutClusters(state.data());
        observe(state, t);
        if ((h.record_every > 0 && k % h.record_every == 0) || k == h.nsteps) dump(state.data(), n3);
      }
    };
    if (h.family == 1) {
      ChimeraSystemPtr system(&thread, h.v0, h.sigma, h.rho, h.alpha,
                              h.D_phi, h.rho_0, pbc_config);
      run_ptr(system);
    } else if (h.family == 2) {
      VortexArraysSystemPtr system(&thread, h.v0, va[0], va[1], va[2], va[3], h.D_phi, va[4], h.rho, pbc_config);
      run_ptr(system);
    } else if (h.family == 0) {
      ChimeraSystem chimera_system(&thread, h.v0, h.sigma, h.rho, h.alpha, h.D_phi, h.rho_0, pbc_config);
      if (h.mode == 1) {
        chimera_system.EvaluateRhs(state, k_prev, k_next, h.k_coef, h.dt);
        dump(k_next.data(), n3);
      } else if (h.mode == 2) {
        std::vector<Real> derivative(n3, 0.0);
        std::vector<std::vector<Real>> additional(kN, std::vector<Real>(2, 0.0));
        chimera_system.EvaluateRhs(state, derivative, additional, h.dt);
        dump(derivative.data(), n3);
        for (int i = 0; i < kN; ++i) dump(additional[i].data(), 2);
      } else {
        if (!noise.empty()) chimera_system.InjectNoise(noise);
        StochasticEulerStepper euler(&thread);
        StochasticRungeKuttaStepper srk(&thread);
        RungeKutta4Stepper rk4(&thread);
        Real t = h.t0;
        if (h.mode == 3 && observer) observer->SaveSystemState(state, t);
        if (device_loop)
          run_device(chimera_system,
                     h.stepper == 0 ? SPC_STEPPER_EULER : h.stepper == 1 ? SPC_STEPPER_SRK : SPC_STEPPER_RK4);
        for (int k = 1; k <= h.nsteps && !device_loop; ++k) {
          t += h.dt;
          if (h.stepper == 0)
            euler.DoStep(chimera_system, state, t, h.dt);
          else if (h.stepper == 1)
            srk.DoStep(chimera_system, state, t, h.dt);
          else
            rk4.DoStep(chimera_system, state, t, h.dt);
          pbc_config.ApplyPeriodicBoundaryConditions(state);
          thread.SynchronizeVector(state);
          observe(state, t);
          if (h.mode == 3 || (h.record_every > 0 && k % h.record_every == 0) || k == h.nsteps)
            dump(state.data(), n3);
        }
      }
    } else {
      std::fprintf(stderr, "spc_dropin_driver: unsupported family/stepper\n");
      return 5;
    }
    delete observer;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  std::fclose(out);
  return 0;
}
