// The drop-in adapters' host logic against the host-memory stand-in of the
// C-ABI (fake_spc.cpp): state shadows, frequencies reaching every handle,
// recovery after a failed step or a throwing observer, and the observer files
// of the device loop against the per-step engine loop.  Prints one line per
// case and exits non-zero on the first failure.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <string>
#include <stdexcept>
#include <vector>

#include "../../spc2_langevin_integration_gb300/host/spc_dropin.hpp"
#include "../../spc2_langevin_integration_gb300/host/spc_observer.hpp"

const int kN = 4;
const Real kL = 1.0;

extern "C" {
void fake_spc_fail_next_step(int after_steps);
long fake_spc_state_uploads(const spc_handle *h);
long fake_spc_omega_uploads(const spc_handle *h);
}

#define CHECK(cond)                                                   \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);     \
      return 1;                                                       \
    }                                                                 \
  } while (0)

namespace {

bool phases_are(const std::vector<Real> &s, Real want) {
  for (int i = 0; i < kN; ++i)
    if (std::fabs(s[3 * i + 2] - want) > 1e-12) return false;
  return true;
}

std::vector<Real> start_state() {
  std::vector<Real> s(3 * kN);
  for (int i = 0; i < kN; ++i) {
    s[3 * i] = 0.1 * i;
    s[3 * i + 1] = 0.2;
    s[3 * i + 2] = 0.5;
  }
  return s;
}

int frequencies_reach_every_handle() {
  Thread th(0, nullptr);
  PeriodicBoundaryConditions pbc(&th, kL, kL);
  VortexArraysSystem sys(&th, 0.01, 1.0, 0.1, 0.0, 1.0, pbc, std::vector<Real>(kN, 1.0));
  std::vector<Real> s = start_state();
  Real t = 0.0;
  sys.Advance(SPC_STEPPER_SRK, s, t, 0.1, 1);    // + 0.1
  sys.Advance(SPC_STEPPER_EULER, s, t, 0.1, 1);  // + 0.1 (second handle)
  CHECK(phases_are(s, 0.7));
  sys.UseFrequencies(std::vector<Real>(kN, 2.0));
  sys.Advance(SPC_STEPPER_SRK, s, t, 0.1, 1);    // + 0.2
  sys.Advance(SPC_STEPPER_EULER, s, t, 0.1, 1);  // + 0.2: the second handle has them too
  CHECK(phases_are(s, 1.1));
  CHECK(fake_spc_omega_uploads(sys.Handle(SPC_STEPPER_SRK)) == 2);
  CHECK(fake_spc_omega_uploads(sys.Handle(SPC_STEPPER_EULER)) == 2);
  // unchanged frequencies are not uploaded again
  sys.UseFrequencies(std::vector<Real>(kN, 2.0));
  sys.Advance(SPC_STEPPER_SRK, s, t, 0.1, 1);
  CHECK(fake_spc_omega_uploads(sys.Handle(SPC_STEPPER_SRK)) == 2);
  std::printf("ok frequencies_reach_every_handle\n");
  return 0;
}

int state_is_uploaded_only_when_it_changed() {
  Thread th(0, nullptr);
  PeriodicBoundaryConditions pbc(&th, kL, kL);
  ChimeraSystem sys(&th, 0.01, 1.0, 0.1, 1.45, 0.0, 1.0, pbc);
  StochasticEulerStepper stepper(&th);
  std::vector<Real> s = start_state();
  stepper.DoStep(sys, s, 0.0, 0.1);
  stepper.DoStep(sys, s, 0.1, 0.1);  // the device already holds s
  spc_handle *h = sys.Handle(SPC_STEPPER_EULER);
  CHECK(fake_spc_state_uploads(h) == 1);
  CHECK(phases_are(s, 0.7));
  s[0] = 0.9;  // the caller edits its state: uploaded before the next step
  stepper.DoStep(sys, s, 0.2, 0.1);
  CHECK(fake_spc_state_uploads(h) == 2);
  CHECK(phases_are(s, 0.8) && s[0] == 0.9);
  std::printf("ok state_is_uploaded_only_when_it_changed\n");
  return 0;
}

int failed_step_reuploads_the_callers_state() {
  Thread th(0, nullptr);
  PeriodicBoundaryConditions pbc(&th, kL, kL);
  ChimeraSystem sys(&th, 0.01, 1.0, 0.1, 1.45, 0.0, 1.0, pbc);
  std::vector<Real> s = start_state();
  Real t = 0.0;
  sys.Advance(SPC_STEPPER_EULER, s, t, 0.1, 1);  // 0.6
  fake_spc_fail_next_step(2);                    // two steps move the device, then an error
  bool threw = false;
  try {
    sys.Advance(SPC_STEPPER_EULER, s, t, 0.1, 3);
  } catch (const std::runtime_error &) {
    threw = true;
  }
  CHECK(threw);
  CHECK(phases_are(s, 0.6) && std::fabs(t - 0.1) < 1e-15);  // the caller's state and time stand
  sys.Advance(SPC_STEPPER_EULER, s, t, 0.1, 1);  // from the caller's state, not the device's
  CHECK(phases_are(s, 0.7));
  CHECK(fake_spc_state_uploads(sys.Handle(SPC_STEPPER_EULER)) == 2);
  std::printf("ok failed_step_reuploads_the_callers_state\n");
  return 0;
}

int throwing_observer_reuploads_the_callers_state() {
  Thread th(0, nullptr);
  PeriodicBoundaryConditions pbc(&th, kL, kL);
  ChimeraSystem sys(&th, 0.01, 1.0, 0.1, 1.45, 0.0, 1.0, pbc);
  std::vector<Real> s = start_state();
  Real t = 0.0;
  std::vector<long> seen;
  // observer on every step: sees steps 1..4, then the run ends normally
  long done = sys.Run(SPC_STEPPER_EULER, s, t, 0.1, 4, 1, {1},
                      [&](long k, Real, const Real *) { seen.push_back(k); return false; });
  CHECK(done == 4 && seen.size() == 4 && seen.back() == 4);
  CHECK(phases_are(s, 0.9));
  // a true return stops the run after that step; state and time follow
  done = sys.Run(SPC_STEPPER_EULER, s, t, 0.1, 10, 1, {1},
                 [&](long k, Real, const Real *) { return k == 2; });
  CHECK(done == 2 && phases_are(s, 1.1) && std::fabs(t - 0.6) < 1e-12);
  bool threw = false;
  try {
    sys.Run(SPC_STEPPER_EULER, s, t, 0.1, 5, 1, {1}, [&](long k, Real, const Real *) -> bool {
      if (k == 3) throw std::runtime_error("observer");
      return false;
    });
  } catch (const std::runtime_error &e) {
    threw = std::string(e.what()) == "observer";
  }
  CHECK(threw);
  CHECK(phases_are(s, 1.1));  // unchanged by the run that threw
  sys.Advance(SPC_STEPPER_EULER, s, t, 0.1, 1);
  CHECK(phases_are(s, 1.2));
  std::printf("ok throwing_observer_reuploads_the_callers_state\n");
  return 0;
}

std::string slurp(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  return std::string(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

// The engine loop of SimulationEngine::RunSimulation (DoStep, then both
// observer calls, every step) against RunObserved on the device loop: the same
// frames and summary lines, byte for byte, at several output thresholds, and
// when the device loop takes over from steps run one at a time.
int observed_loop_writes_the_per_step_files() {
  const int thresholds[][2] = {{1, 1}, {3, 2}, {10, 10}, {4, 6}};
  int trial = 0;
  for (const auto &th2 : thresholds) {
    Thread th(0, nullptr);
    PeriodicBoundaryConditions pbc(&th, kL, kL);
    ChimeraSystem a(&th, 0.01, 1.0, 0.1, 1.45, 0.0, 1.0, pbc), b(&th, 0.01, 1.0, 0.1, 1.45, 0.0, 1.0, pbc);
    StochasticEulerStepper stepper(&th);
    BinaryObserver oa(&th, 0.01, 1.0, 0.1, 1.45, 0.0, 1.0, pbc, 0.1, 2 * trial);
    BinaryObserver ob(&th, 0.01, 1.0, 0.1, 1.45, 0.0, 1.0, pbc, 0.1, 2 * trial + 1);
    ++trial;
    oa.SetOutputThresholds(th2[0], th2[1]);
    ob.SetOutputThresholds(th2[0], th2[1]);
    std::vector<Real> sa = start_state(), sb = start_state();
    Real ta = 0.0, tb = 0.0;
    const Real dt = 0.1;
    for (int k = 0; k < 28; ++k) {  // the reference's loop
      stepper.DoStep(a, sa, ta, dt);
      ta += dt;
      oa.SaveSystemState(sa, ta);
      oa.SaveSummaryStatistics(sa, ta);
    }
    for (int k = 0; k < 5; ++k) {  // five steps one at a time, then the device loop
      stepper.DoStep(b, sb, tb, dt);
      tb += dt;
      ob.SaveSystemState(sb, tb);
      ob.SaveSummaryStatistics(sb, tb);
    }
    RunObserved(b, SPC_STEPPER_EULER, sb, tb, dt, 23, &ob);
    CHECK(sa == sb && std::fabs(ta - tb) < 1e-12);
    // one more call of each after the device loop: the counters must agree too
    oa.SaveSystemState(sa, ta);
    oa.SaveSummaryStatistics(sa, ta);
    ob.SaveSystemState(sb, tb);
    ob.SaveSummaryStatistics(sb, tb);
    const std::string fa = slurp(oa.SimulationFileName()), fb = slurp(ob.SimulationFileName());
    const std::string qa = slurp(oa.SummaryStatisticsFileName()), qb = slurp(ob.SummaryStatisticsFileName());
    CHECK(!fa.empty() && fa == fb);
    CHECK(!qa.empty() && qa == qb);
    // frames written: ceil(29 / threshold), each 4 bytes of time + 3N float32
    CHECK(fa.size() == (size_t)((29 + th2[0] - 1) / th2[0]) * (1 + 3 * kN) * 4);
  }
  std::printf("ok observed_loop_writes_the_per_step_files\n");
  return 0;
}

}  // namespace

int main() {
  if (frequencies_reach_every_handle()) return 1;
  if (state_is_uploaded_only_when_it_changed()) return 1;
  if (failed_step_reuploads_the_callers_state()) return 1;
  if (throwing_observer_reuploads_the_callers_state()) return 1;
  if (observed_loop_writes_the_per_step_files()) return 1;
  return 0;
}
