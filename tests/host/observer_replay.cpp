// Replays a recorded trajectory through the drop-in's BinaryObserver
// (host/spc_observer.cpp) the way the reference's engine loop drives its own
// (SimulationEngine.cpp:113-127): the frame of the initial state at t0, then
// after every step the frame and the summary line.  The caller compares the
// files it writes (into SPC_OUTPUT_DIR) with the reference observer's.
//
// usage: SPC_N=<N> SPC_OUTPUT_DIR=<dir> observer_replay <input.bin>
// input (little endian): int32 nsteps, pad; double L, t0, dt, v0, sigma, rho,
// alpha, D_phi, rho_0; double state0[3N]; double states[nsteps][3N].
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../spc2_langevin_integration_gb300/host/spc_dropin.hpp"
#include "../../spc2_langevin_integration_gb300/host/spc_observer.hpp"

static int env_n() {
  const char *v = std::getenv("SPC_N");
  return v ? std::atoi(v) : 0;
}
extern const int kN = env_n();
extern const Real kL = 1.0;  // the observer does not use the box

int main(int argc, char **argv) {
  if (argc != 2 || kN <= 0) {
    std::fprintf(stderr, "usage: SPC_N=<N> observer_replay <input.bin>\n");
    return 2;
  }
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t hdr[2];
  double prm[9];
  if (std::fread(hdr, sizeof(hdr), 1, f) != 1 || std::fread(prm, sizeof(prm), 1, f) != 1) return 2;
  const int nsteps = hdr[0];
  const size_t n3 = (size_t)kS * kN;
  std::vector<Real> state(n3);
  Thread thread(argc, argv);
  PeriodicBoundaryConditions pbc(&thread, prm[0], prm[0]);
  BinaryObserver observer(&thread, prm[3], prm[4], prm[5], prm[6], prm[7], prm[8], pbc, prm[2], 0);
  if (std::fread(state.data(), sizeof(Real), n3, f) != n3) return 2;
  Real t = prm[1];
  observer.SaveSystemState(state, t);
  for (int k = 1; k <= nsteps; ++k) {
    if (std::fread(state.data(), sizeof(Real), n3, f) != n3) return 2;
    t += prm[2];
    observer.SaveSystemState(state, t);
    observer.SaveSummaryStatistics(state, t);
  }
  std::fclose(f);
  return 0;
}
