// Driver that runs the reference's own particle-update code (compiled from its
// unmodified sources with oracle/ref/ref_prelude.hpp force-included) on an
// injected input, for the oracle's golden vectors.  Test infrastructure only.
//
// usage: SPC_REF_N=<N> SPC_REF_L=<L> spc_ref <input.bin> <output.bin>
//
// input (little endian):
//   char[8] "SPCREF01"; int32 mode, family, stepper, nsteps, record_every, pad;
//   double v0, sigma, rho, alpha, D_phi, rho_0, t0, dt, k_coef;
//   double state[3N], k_prev[3N], k_next_init[3N];
//   int64 n_noise; double noise[n_noise]   (consumed in the reference's draw order)
// mode 0 = run the engine loop (SimulationEngine.cpp:149-161 / SimulationEnginePtr.cpp:106-115)
//          nsteps times and write the state every record_every steps (and at the end);
// mode 1 = one RK-form EvaluateRhs -> k_next[3N];
// mode 2 = one SRK-form EvaluateRhs -> derivative[3N] then additional[2N] ([i][0], [i][1]);
// mode 3 = the engine loop of SimulationEngine.cpp:113-127 with the reference's
//          BinaryObserver (family 0): the initial frame at t0, then after every
//          step the frame and the summary line, into SPC_REF_OUT_DIR; every
//          state after a step is written to the output.
// family 0 = vector classes (Thread, ChimeraSystem, *Stepper);
// family 1 = shared-window classes (ThreadSharedMemory, ChimeraSystemPtr, *StepperPtr);
// family 2 = VortexArraysSystemPtr with the *StepperPtr classes; its five extra
//            parameters follow the noise block: double mu_plus, mu_minus, xi_a,
//            xi_r, kappa (velocity = v0, rho, D_phi from the header).
// stepper 0 = StochasticEuler, 1 = StochasticRungeKutta, 2 = RungeKutta4.
#include "Parallelization/Thread.hpp"
#include "Parallelization/ThreadSharedMemory.hpp"
#include "BoundaryConfiguration/PeriodicBoundaryConditions.hpp"
#include "DynamicalSystems/ChimeraSystem.hpp"
#include "DynamicalSystems/ChimeraSystemPtr.hpp"
#include "DynamicalSystems/VortexArraysSystemPtr.hpp"
#include "Steppers/StochasticEulerStepper.hpp"
#include "Steppers/StochasticRungeKuttaStepper.hpp"
#include "Steppers/RungeKutta4Stepper.hpp"
#include "Steppers/StochasticEulerStepperPtr.hpp"
#include "Steppers/StochasticRungeKuttaStepperPtr.hpp"
#include "Steppers/RungeKutta4StepperPtr.hpp"
#include "Observers/BinaryObserver.hpp"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static int env_int(const char *k) {
  const char *v = std::getenv(k);
  if (!v) {
    std::fprintf(stderr, "spc_ref: %s is not set\n", k);
    std::exit(2);
  }
  return std::atoi(v);
}
static double env_double(const char *k) {
  const char *v = std::getenv(k);
  if (!v) {
    std::fprintf(stderr, "spc_ref: %s is not set\n", k);
    std::exit(2);
  }
  return std::strtod(v, nullptr);
}

extern const int kN = env_int("SPC_REF_N");
extern const Real kL = env_double("SPC_REF_L");
std::mt19937 mersenne_twister_generator(0u);

namespace spc_ref {
static std::vector<double> g_noise;
static std::size_t g_pos = 0;
double next_injected_normal() {
  if (g_pos >= g_noise.size()) {
    std::fprintf(stderr, "spc_ref: injected noise stream exhausted at %zu\n", g_pos);
    std::exit(3);
  }
  return g_noise[g_pos++];
}

// BinaryObserver's output folder (see ref_prelude.hpp): SPC_REF_OUT_DIR.
const char *output_folder(const char *) {
  static std::string folder;
  const char *d = std::getenv("SPC_REF_OUT_DIR");
  if (!d) {
    std::fprintf(stderr, "spc_ref: SPC_REF_OUT_DIR is not set\n");
    std::exit(2);
  }
  folder = std::string(d) + "/";
  return folder.c_str();
}
}  // namespace spc_ref

struct Header {
  char magic[8];
  int32_t mode, family, stepper, nsteps, record_every, pad;
  double v0, sigma, rho, alpha, D_phi, rho_0, t0, dt, k_coef;
};

static void read_exact(FILE *f, void *p, std::size_t n) {
  if (std::fread(p, 1, n, f) != n) {
    std::fprintf(stderr, "spc_ref: short input\n");
    std::exit(2);
  }
}

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: spc_ref <input.bin> <output.bin>\n");
    return 2;
  }
  FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  Header h;
  read_exact(in, &h, sizeof(h));
  if (std::memcmp(h.magic, "SPCREF01", 8) != 0) {
    std::fprintf(stderr, "spc_ref: bad magic\n");
    return 2;
  }
  const std::size_t n3 = (std::size_t)kS * kN;
  std::vector<Real> state(n3), k_prev(n3), k_next(n3);
  read_exact(in, state.data(), n3 * sizeof(Real));
  read_exact(in, k_prev.data(), n3 * sizeof(Real));
  read_exact(in, k_next.data(), n3 * sizeof(Real));
  int64_t n_noise = 0;
  read_exact(in, &n_noise, sizeof(n_noise));
  spc_ref::g_noise.resize((std::size_t)n_noise);
  if (n_noise) read_exact(in, spc_ref::g_noise.data(), (std::size_t)n_noise * sizeof(double));
  double va[5] = {0, 0, 0, 0, 0};
  if (h.family == 2) read_exact(in, va, sizeof(va));
  std::fclose(in);

  FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  auto dump = [&](const Real *p, std::size_t n) { std::fwrite(p, sizeof(Real), n, out); };

  if (h.family == 0) {
    Thread thread(argc, argv);
    PeriodicBoundaryConditions pbc(&thread, kL, kL);
    ChimeraSystem system(&thread, h.v0, h.sigma, h.rho, h.alpha, h.D_phi, h.rho_0, pbc);
    if (h.mode == 1) {
      system.EvaluateRhs(state, k_prev, k_next, h.k_coef, h.dt);
      dump(k_next.data(), n3);
    } else if (h.mode == 2) {
      std::vector<Real> derivative(n3, 0.0);
      std::vector<std::vector<Real>> additional(kN, std::vector<Real>(2, 0.0));
      system.EvaluateRhs(state, derivative, additional, h.dt);
      dump(derivative.data(), n3);
      for (int i = 0; i < kN; ++i) dump(additional[i].data(), 2);
    } else if (h.mode == 3) {
      StochasticEulerStepper euler(&thread);
      StochasticRungeKuttaStepper srk(&thread);
      RungeKutta4Stepper rk4(&thread);
      BinaryObserver observer(&thread, h.v0, h.sigma, h.rho, h.alpha, h.D_phi, h.rho_0, pbc, h.dt, 0);
      Real t = h.t0;
      observer.SaveSystemState(state, t);
      for (int k = 1; k <= h.nsteps; ++k) {
        t += h.dt;
        if (h.stepper == 0)
          euler.DoStep(system, state, t, h.dt);
        else if (h.stepper == 1)
          srk.DoStep(system, state, t, h.dt);
        else
          rk4.DoStep(system, state, t, h.dt);
        pbc.ApplyPeriodicBoundaryConditions(state);
        observer.SaveSystemState(state, t);
        observer.SaveSummaryStatistics(state, t);
        dump(state.data(), n3);
      }
    } else {
      StochasticEulerStepper euler(&thread);
      StochasticRungeKuttaStepper srk(&thread);
      RungeKutta4Stepper rk4(&thread);
      Real t = h.t0;
      for (int k = 1; k <= h.nsteps; ++k) {
        t += h.dt;
        if (h.stepper == 0)
          euler.DoStep(system, state, t, h.dt);
        else if (h.stepper == 1)
          srk.DoStep(system, state, t, h.dt);
        else
          rk4.DoStep(system, state, t, h.dt);
        pbc.ApplyPeriodicBoundaryConditions(state);
        if ((h.record_every > 0 && k % h.record_every == 0) || k == h.nsteps)
          dump(state.data(), n3);
      }
    }
  } else if (h.family == 2) {
    ThreadSharedMemory thread(argc, argv);
    PeriodicBoundaryConditions pbc(&thread, kL, kL);
    {
      VortexArraysSystemPtr system(&thread, h.v0, va[0], va[1], va[2], va[3], h.D_phi, va[4], h.rho, pbc);
      if (h.mode == 1) {
        system.EvaluateRhs(state.data(), k_prev, k_next, h.k_coef, h.dt);
        dump(k_next.data(), n3);
      } else if (h.mode == 2) {
        std::vector<Real> derivative(n3, 0.0);
        std::vector<std::vector<Real>> additional(kN, std::vector<Real>(2, 0.0));
        system.EvaluateRhs(state.data(), derivative, additional, h.dt);
        dump(derivative.data(), n3);
        for (int i = 0; i < kN; ++i) dump(additional[i].data(), 2);
      } else {
        // the SRK-Ptr constructor draws N natural frequencies first, which the
        // vortex-arrays update does not use
        StochasticRungeKuttaStepperPtr *srk =
            h.stepper == 1 ? new StochasticRungeKuttaStepperPtr(&thread) : nullptr;
        StochasticEulerStepperPtr euler(&thread);
        RungeKutta4StepperPtr rk4(&thread);
        Real t = h.t0;
        for (int k = 1; k <= h.nsteps; ++k) {
          t += h.dt;
          if (h.stepper == 0)
            euler.DoStep(system, state.data(), t, h.dt);
          else if (h.stepper == 1)
            srk->DoStep(system, state.data(), t, h.dt);
          else
            rk4.DoStep(system, state.data(), t, h.dt);
          pbc.ApplyPeriodicBoundaryConditions(state.data(), (long)n3);
          if ((h.record_every > 0 && k % h.record_every == 0) || k == h.nsteps)
            dump(state.data(), n3);
        }
        delete srk;
      }
    }
  } else {
    ThreadSharedMemory thread(argc, argv);
    PeriodicBoundaryConditions pbc(&thread, kL, kL);
    {
      ChimeraSystemPtr system(&thread, h.v0, h.sigma, h.rho, h.alpha, h.D_phi, h.rho_0, pbc);
      if (h.mode == 1) {
        system.EvaluateRhs(state.data(), k_prev, k_next, h.k_coef, h.dt);
        dump(k_next.data(), n3);
      } else if (h.mode == 2) {
        std::vector<Real> derivative(n3, 0.0);
        std::vector<std::vector<Real>> additional(kN, std::vector<Real>(2, 0.0));
        system.EvaluateRhs(state.data(), derivative, additional, h.dt);
        dump(derivative.data(), n3);
        for (int i = 0; i < kN; ++i) dump(additional[i].data(), 2);
      } else {
        // The SRK-Ptr constructor draws the natural frequencies first
        // (StochasticRungeKuttaStepperPtr.hpp:30-34): the first N injected
        // values are omega.
        StochasticRungeKuttaStepperPtr *srk =
            h.stepper == 1 ? new StochasticRungeKuttaStepperPtr(&thread) : nullptr;
        StochasticEulerStepperPtr euler(&thread);
        RungeKutta4StepperPtr rk4(&thread);
        Real t = h.t0;
        for (int k = 1; k <= h.nsteps; ++k) {
          t += h.dt;
          if (h.stepper == 0)
            euler.DoStep(system, state.data(), t, h.dt);
          else if (h.stepper == 1)
            srk->DoStep(system, state.data(), t, h.dt);
          else
            rk4.DoStep(system, state.data(), t, h.dt);
          pbc.ApplyPeriodicBoundaryConditions(state.data(), (long)n3);
          if ((h.record_every > 0 && k % h.record_every == 0) || k == h.nsteps)
            dump(state.data(), n3);
        }
        delete srk;
      }
    }
  }
  std::fclose(out);
  if (spc_ref::g_pos != spc_ref::g_noise.size()) {
    std::fprintf(stderr, "spc_ref: %zu of %zu injected normals unused\n",
                 spc_ref::g_noise.size() - spc_ref::g_pos, spc_ref::g_noise.size());
    return 4;
  }
  return 0;
}
