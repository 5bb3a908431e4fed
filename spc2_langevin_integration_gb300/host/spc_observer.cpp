// Observers and restart reader in the reference's file formats (spc_observer.hpp).
#include "spc_observer.hpp"

#include <cmath>
#include <complex>
#include <numeric>
#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <stdexcept>

namespace {

std::string output_folder() {
  const char *d = std::getenv("SPC_OUTPUT_DIR");
  std::string f = d ? d : ".";
  if (!f.empty() && f.back() != '/') f += '/';
  return f;
}

std::string parameter_tag(Real v_0, Real sigma, Real rho, Real alpha, Real D_phi, Real rho_0, int trial) {
  // the reference's pattern (BinaryObserver.cpp:47-55), default stream formatting
  std::ostringstream b;
  b << "v0_" << v_0 << "_sigma_" << sigma << "_rho_" << rho << "_alpha_" << alpha << "_Dphi_" << D_phi
    << "_N_" << kN << "_rho0_" << rho_0 << "_" << 0 << "_" << trial;
  return b.str();
}

}  // namespace

BinaryObserver::BinaryObserver(Thread *thread, Real v_0, Real sigma, Real rho, Real alpha, Real D_phi,
                               Real rho_0, PeriodicBoundaryConditions &, Real, int trial)
    : thread_(thread), frame_((size_t)kS * kN, 0.0f) {
  if (!thread_->IsRoot()) return;
  const std::string tag = parameter_tag(v_0, sigma, rho, alpha, D_phi, rho_0, trial);
  simulation_file_name_ = output_folder() + tag + ".bin";
  summary_statistics_file_name_ = output_folder() + "summary_statistics_" + tag + ".txt";
  std::remove(simulation_file_name_.c_str());
  std::remove(summary_statistics_file_name_.c_str());
  simulation_file_.open(simulation_file_name_, std::ios::binary | std::ios::out | std::ios::app);
  summary_statistics_file_.open(summary_statistics_file_name_, std::ios::out | std::ios::app);
  if (!simulation_file_.is_open() || !summary_statistics_file_.is_open())
    throw std::runtime_error("BinaryObserver: cannot open output files in " + output_folder());
}

BinaryObserver::~BinaryObserver() {
  if (simulation_file_.is_open()) simulation_file_.close();
  if (summary_statistics_file_.is_open()) summary_statistics_file_.close();
}

void BinaryObserver::SetOutputThresholds(int state_every, int summary_every) {
  if (state_every < 1 || summary_every < 1) throw std::invalid_argument("thresholds must be >= 1");
  output_time_threshold_[0] = state_every;
  output_time_threshold_[1] = summary_every;
}

void BinaryObserver::SaveSystemState(std::vector<Real> &system_state, Real t) {
  if (thread_->IsRoot() && !(output_time_counter_[0] % output_time_threshold_[0])) {
    const float t_float = (float)t;
    for (size_t i = 0; i < frame_.size(); ++i) frame_[i] = (float)system_state[i];
    simulation_file_.write(reinterpret_cast<const char *>(&t_float), sizeof(float));
    simulation_file_.write(reinterpret_cast<const char *>(frame_.data()), frame_.size() * sizeof(float));
    simulation_file_.flush();
  }
  ++output_time_counter_[0];
}

void BinaryObserver::SaveSummaryStatistics(std::vector<Real> &system_state, Real t) {
  if (thread_->IsRoot() && !(output_time_counter_[1] % output_time_threshold_[1])) {
    const float t_float = (float)t;
    std::complex<float> r(0.0f, 0.0f);
    for (int i = 0; i < kN; ++i) {
      const Real phi = system_state[(size_t)kS * i + 2];
      r += std::complex<float>((float)std::cos(phi), (float)std::sin(phi));
    }
    r /= (float)kN;
    summary_statistics_file_ << t_float << '\t' << std::abs(r) << '\t' << std::arg(r) << std::endl;
  }
  ++output_time_counter_[1];
}

void InitializeSystemStateFromFile(const std::string &file_name, std::vector<Real> &system_state) {
  std::ifstream f(file_name, std::ios::binary | std::ios::in);
  if (!f.is_open()) throw std::runtime_error("cannot open " + file_name);
  std::vector<float> buf((size_t)kS * kN, 0.0f);
  f.read(reinterpret_cast<char *>(buf.data()), (std::streamsize)(buf.size() * sizeof(float)));
  if ((size_t)f.gcount() != buf.size() * sizeof(float))
    throw std::runtime_error(file_name + ": fewer than 3N float32 values");
  system_state.assign(buf.begin(), buf.end());
}

bool BinaryObserver::StateWrittenAt(long j) const {
  const long T = output_time_threshold_[0];
  return thread_->IsRoot() && ((output_time_counter_[0] + j - 1) % T + T) % T == 0;
}

bool BinaryObserver::SummaryWrittenAt(long j) const {
  const long T = output_time_threshold_[1];
  return thread_->IsRoot() && ((output_time_counter_[1] + j - 1) % T + T) % T == 0;
}

void BinaryObserver::SkipCalls(long n) {
  output_time_counter_[0] += (int)n;
  output_time_counter_[1] += (int)n;
}

long BinaryObserver::CadencePeriod() const {
  const long a = output_time_threshold_[0], b = output_time_threshold_[1];
  return a / std::gcd(a, b) * b;
}

void RunObserved(SpcSystemBase &system, int stepper, std::vector<Real> &state, Real &t, Real dt, long nsteps,
                 BinaryObserver *observer, long every,
                 const std::function<void(long, Real, const std::vector<Real> &)> &on_state) {
  long period = observer ? observer->CadencePeriod() : 1;
  if (every > 0) period = period / std::gcd(period, every) * every;
  if (period > (1L << 20)) throw std::runtime_error("RunObserved: observer cadence period too long");
  // step k is observed when k % period == j: j stands for step j (or period)
  std::vector<uint8_t> observe((size_t)period, 0);
  for (long j = 0; j < period; ++j) {
    const long k = j == 0 ? period : j;
    observe[(size_t)j] = (observer && (observer->StateWrittenAt(k) || observer->SummaryWrittenAt(k))) ||
                         (every > 0 && k % every == 0);
  }
  std::vector<Real> snapshot;
  long last = 0;
  auto fn = [&](long k, Real tk, const Real *s) {
    snapshot.assign(s, s + (size_t)kS * kN);
    if (observer) {
      observer->SkipCalls(k - last - 1);
      observer->SaveSystemState(snapshot, tk);
      observer->SaveSummaryStatistics(snapshot, tk);
    }
    if (every > 0 && k % every == 0 && on_state) on_state(k, tk, snapshot);
    last = k;
    return false;
  };
  const long done = system.Run(stepper, state, t, dt, nsteps, (int)period, observe, fn);
  if (observer) observer->SkipCalls(done - last);
}
