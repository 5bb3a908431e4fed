// Observers and restart reader in the reference's file formats, for programs
// that use the drop-in classes (spc_dropin.hpp).
//
// BinaryObserver (Observers/BinaryObserver.hpp:15-60):
//  * SaveSystemState appends one frame to <...>.bin: the time as float32, then
//    the 3N state values as float32 in array-of-structures order
//    (BinaryObserver.cpp:186-191);
//  * SaveSummaryStatistics appends "t<TAB>|R|<TAB>arg R<NEWLINE>" to
//    summary_statistics_<...>.txt, R = (1/N) sum_i (cos phi_i, sin phi_i)
//    accumulated in complex<float> in index order (BinaryObserver.cpp:196-234);
//  * each writes on every threshold-th call (the reference's counters, both 1).
// File names follow the reference's pattern ("v0_<v0>_sigma_<sigma>_rho_<rho>
// _alpha_<alpha>_Dphi_<D>_N_<N>_rho0_<rho0>_0_<trial>"); the folder, which the
// reference hard-codes per machine, is $SPC_OUTPUT_DIR (default: the working
// directory).  Output is byte-for-byte what the reference writes for the same
// state and time.
// InitializeSystemStateFromFile (SimulationEngine.cpp:52-73): 3N float32 read
// from the start of a file into the double state.
#pragma once

#include <fstream>
#include <functional>
#include <string>
#include <vector>

#include "spc_dropin.hpp"

class BinaryObserver {
 public:
  BinaryObserver(Thread *thread, Real v_0, Real sigma, Real rho, Real alpha, Real D_phi, Real rho_0,
                 PeriodicBoundaryConditions &pbc_config, Real dt, int trial);
  ~BinaryObserver();

  void SaveSystemState(std::vector<Real> &system_state, Real t);
  void SaveSummaryStatistics(std::vector<Real> &system_state, Real t);

  // write every `state_every`-th / `summary_every`-th call (the reference's
  // output_time_threshold_, 1 and 1 there)
  void SetOutputThresholds(int state_every, int summary_every);
  // the device loop (RunObserved): whether the j-th next call (j >= 1) of
  // SaveSystemState / SaveSummaryStatistics writes, and n calls of each that
  // write nothing (the counters advance as if the engine had called them)
  bool StateWrittenAt(long j) const;
  bool SummaryWrittenAt(long j) const;
  void SkipCalls(long n);
  long CadencePeriod() const;  // lcm of the two thresholds
  const std::string &SimulationFileName() const { return simulation_file_name_; }
  const std::string &SummaryStatisticsFileName() const { return summary_statistics_file_name_; }

 private:
  Thread *thread_;
  int output_time_counter_[2] = {0, 0};
  int output_time_threshold_[2] = {1, 1};
  std::string simulation_file_name_, summary_statistics_file_name_;
  std::ofstream simulation_file_, summary_statistics_file_;
  std::vector<float> frame_;
};

void InitializeSystemStateFromFile(const std::string &file_name, std::vector<Real> &system_state);

// The engine loop of SimulationEngine::RunSimulation (SimulationEngine.cpp:149-161)
// for nsteps steps of stepper kind `stepper`, run on the device by spc_run:
// the observer writes exactly the frames and summary lines its counters ask
// for, from snapshots of those steps, while the device runs the next steps.
// With every > 0, on_state also sees the state after every every-th step.
// state and t end as after the last step.
void RunObserved(SpcSystemBase &system, int stepper, std::vector<Real> &state, Real &t, Real dt, long nsteps,
                 BinaryObserver *observer, long every = 0,
                 const std::function<void(long, Real, const std::vector<Real> &)> &on_state = nullptr);
