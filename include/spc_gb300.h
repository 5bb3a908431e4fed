/*
 * spc_gb300.h -- C-ABI of the GB300 (sm_103a) particle-update library.
 *
 * The reference (raven91/spc2_langevin_integration) has no FFI: its "plugin"
 * surface is the C++ stepper/system contract
 *   Stepper::DoStep(System&, std::vector<Real>& state, Real t, Real dt)
 *   System::EvaluateRhs(state, k_prev, k_next, k_coef, dt)            (RK form)
 *   System::EvaluateRhs(state, derivative, additional_derivative, dt)  (SRK form)
 * plus the engine's PeriodicBoundaryConditions wrap.  This header is the thin,
 * allocation-owning C layer those classes forward to (the C++ adapters in
 * spc2_langevin_integration_gb300/host keep the reference class names and
 * signatures).  Each entry point names the reference interface it replaces.
 *
 * Conventions: every function returns 0 (SPC_OK) or a negative spc_status;
 * spc_last_error() gives a message.  State crosses the boundary in the
 * reference's array-of-structures layout [x0,y0,phi0,x1,...] (3N doubles);
 * on the device it is structure-of-arrays.  A handle is used from one host
 * thread at a time and owns one CUDA stream and all of its device memory.
 */
#ifndef SPC_GB300_H
#define SPC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPC_ABI_VERSION 4

typedef enum spc_status {
  SPC_OK = 0,
  SPC_ERR_INVALID = -1,   /* bad argument or parameter */
  SPC_ERR_CUDA = -2,      /* a CUDA call failed (message has the CUDA error) */
  SPC_ERR_NOMEM = -3,     /* device allocation failed */
  SPC_ERR_STATE = -4,     /* call out of order (e.g. stepping before upload) */
  SPC_ERR_NOISE = -5,     /* injected noise stream exhausted */
  SPC_ERR_DEVICE = -6,    /* a kernel reported an error word (see message) */
  SPC_ERR_CAPACITY = -7   /* a caller-provided buffer is too small */
} spc_status;

/* Dynamical system.  CHIMERA: ChimeraSystem (DynamicalSystems/ChimeraSystem.hpp:12-106).
 * VORTEX: the same alignment right-hand side with per-particle natural
 * frequencies omega_i added to the phase drift of the stochastic
 * Runge-Kutta update, as StochasticRungeKuttaStepperPtr does
 * (Steppers/StochasticRungeKuttaStepperPtr.hpp:27-34, :65). */
enum { SPC_MODEL_CHIMERA = 0, SPC_MODEL_VORTEX = 1, SPC_MODEL_VORTEX_ARRAYS = 2 };
/* VORTEX_ARRAYS: VortexArraysSystemPtr (DynamicalSystems/VortexArraysSystemPtr.cpp),
 * velocity v0, distance-dependent alignment mu_plus (1 - r^2/xi_a^2) inside
 * xi_a and anti-alignment -4 mu_minus (r - xi_a)(rho - r)/(rho - xi_a)^2 up to
 * rho (:737-763), cohesion -kappa sin(atan2(dy, dx) - phi_i) inside xi_r, and
 * its heavier stochastic Runge-Kutta second pass (:659-732).  Plain FP64 only;
 * steppers EULER_PTR, SRK and RK4 (the *StepperPtr forms the reference pairs it
 * with); the cell-list search (or all pairs when rho > L/4). */

/* Stepper.  EULER: StochasticEulerStepper (Steppers/StochasticEulerStepper.hpp:31-47);
 * SRK: StochasticRungeKuttaStepper(Ptr) strong order 1.5
 * (Steppers/StochasticRungeKuttaStepper.hpp:34-61); RK4: RungeKutta4Stepper
 * (Steppers/RungeKutta4Stepper.cpp:29-57); EULER_PTR: StochasticEulerStepperPtr
 * (Steppers/StochasticEulerStepperPtr.hpp:32-53). */
enum { SPC_STEPPER_EULER = 0, SPC_STEPPER_SRK = 1, SPC_STEPPER_RK4 = 2, SPC_STEPPER_EULER_PTR = 3 };

/* Neighbour search.  CELL: the reference's linked-list cells of side
 * L/int(L/rho) and 3x3 stencil (ChimeraSystem.cpp:258-426).  VERLET: a
 * skin list (r_max = rho + skin) rebuilt when the largest displacement since
 * the last build exceeds skin/2; its neighbour sets equal the cell search's.
 * When rho > L/4 both fall back to all pairs, as EvaluateRhs does
 * (ChimeraSystem.cpp:90-98). */
enum { SPC_NEIGHBOUR_CELL = 0, SPC_NEIGHBOUR_VERLET = 1 };

/* Precision.  FP64: every value and operation in double, in the reference's
 * order.  FP32C: neighbour sums, sin/cos and stage updates in float with
 * compensated (Kahan) accumulation; the cutoff / minimum-image decision, the
 * wrapped positions and the accumulated phase stay double.
 * FP32X: the per-pair work stays off the FP64 pipe (float prefilter, the
 * exact FP64 test only near the cutoff), and the neighbour sums are exact:
 * each particle's cos phi and sin phi (and, for the SRK second pass, the
 * same weighted by its phase rate) are rounded once to 64-bit fixed point
 * (2^-52 resolution) and summed as integers, which is exact and independent
 * of order.  The per-particle work (sin/cos, the angle-addition identity
 * sin(phi_j - phi_i - alpha) = sin phi_j cos(phi_i + alpha) - cos phi_j
 * sin(phi_i + alpha), the stepper update and the noise) is FP64 with the
 * plain form's formulas and normals, so results follow the FP64 form to a
 * few 1e-16 relative per right-hand side.  Cell list and all pairs only
 * (SPC_NEIGHBOUR_VERLET is refused); the Chimera and vortex models. */
enum { SPC_PRECISION_FP64 = 0, SPC_PRECISION_FP32C = 1, SPC_PRECISION_FP32X = 2 };

/* flags */
#define SPC_FLAG_EXACT_ALL 0x1u /* decide every candidate pair in FP64 (no float prefilter) */

typedef struct spc_params {
  int32_t model;      /* SPC_MODEL_* */
  int32_t stepper;    /* SPC_STEPPER_* */
  int32_t neighbour;  /* SPC_NEIGHBOUR_* */
  int32_t precision;  /* SPC_PRECISION_* */
  double L;           /* periodic box side (kL, Definitions.hpp:22) */
  double v0, sigma, rho, alpha, D_phi, rho_0; /* ChimeraSystem ctor (ChimeraSystem.hpp:16-23) */
  double skin;        /* Verlet skin; r_max = rho + skin */
  uint64_t seed;      /* Philox4x32-10 key */
  uint32_t system_id; /* Philox counter word: distinguishes systems sharing a seed */
  uint32_t flags;     /* SPC_FLAG_* */
  /* VORTEX_ARRAYS only (VortexArraysSystemPtr ctor, VortexArraysSystemPtr.cpp:9-18) */
  double mu_plus, mu_minus, xi_a, xi_r, kappa;
} spc_params;

typedef struct spc_handle spc_handle;

/* Library / version.  SPC_ABI_VERSION changes with any layout change of the
 * structs above or below (3: spc_tuning gained cell_units; 4: subcells). */
int spc_abi_version(void);
const char *spc_last_error(const spc_handle *h); /* h may be NULL: last global error */

/* Construct a system of n particles (replaces the ChimeraSystem ctor
 * ChimeraSystem.cpp:11-59 + the stepper ctors + PeriodicBoundaryConditions
 * ctor PeriodicBoundaryConditions.cpp:7-17).  Allocates all device memory. */
int spc_create(const spc_params *p, int32_t n, spc_handle **out);
int spc_destroy(spc_handle *h);
int spc_get_params(const spc_handle *h, spc_params *out, int32_t *n);

/* State transfer in the reference's AoS layout (replaces the engine's
 * system_state_ vector, SimulationEngine.hpp:27, and BroadcastVector). */
int spc_upload_state(spc_handle *h, const double *aos3n);
int spc_download_state(spc_handle *h, double *aos3n);
/* Natural frequencies (VORTEX model), n doubles
 * (StochasticRungeKuttaStepperPtr.hpp:27-34 frequencies_). */
int spc_upload_omega(spc_handle *h, const double *omega);
/* RK4 stage buffers k1..k4 (4 x 3N, AoS each), which persist across steps
 * (RungeKutta4Stepper.cpp:7-13); for exact resume and tests. */
int spc_download_rk4_buffers(spc_handle *h, double *out12n);
int spc_upload_rk4_buffers(spc_handle *h, const double *in12n);

/* Advance nsteps steps: for each, t += dt; Stepper::DoStep; the engine's
 * periodic wrap (SimulationEngine.cpp:149-155), fused on the device.
 * Noise comes from Philox4x32-10 (counter = particle, system, step) unless an
 * injected stream is set.  *t_inout is advanced. */
int spc_step(spc_handle *h, double *t_inout, double dt, int32_t nsteps);
/* Same, captured as a CUDA graph of nsteps steps on first use and replayed
 * (fixed-length step loops; requires Philox noise). */
int spc_step_graph(spc_handle *h, double *t_inout, double dt, int32_t nsteps);
/* Capture the graph spc_step_graph(h, ., dt, nsteps) replays, without
 * launching it (no counterpart in the reference): after a change that drops
 * the cached graph (a tuning change, a new handle), the capture cost then
 * falls here instead of inside the next timed or latency-bound call.  State
 * and step counter are untouched. */
int spc_prepare_graph(spc_handle *h, double dt, int32_t nsteps);

/* The engine loop with its observers, on the device
 * (SimulationEngine.cpp:149-161, SimulationEnginePtr.cpp:106-115): nsteps
 * steps from *t_inout, and after the k-th of them (k = 1..nsteps) a snapshot
 * of the state when observe[k % period] is nonzero.  A snapshot holds 3N
 * doubles (AoS), exactly what spc_download_state returns after that step.
 * fn(user, k, t_k, state) is called for every snapshot in order of k, with t_k
 * = *t_inout plus dt added k times (SimulationEngine.cpp:151), from the
 * calling thread while the device runs later steps; the pointer is valid
 * during the call only.  A nonzero return from fn stops the run: no later
 * snapshot is delivered, the steps already enqueued (at most one chunk of
 * about 64 steps) complete, and *steps_done (if not NULL) says how many steps
 * the state advanced; *t_inout is the time after them.  Chunks run as CUDA
 * graph replays under Philox noise and eagerly with injected noise; their
 * snapshots reach the host in one copy per chunk on a second stream.  fn may
 * be NULL (no snapshots; observe is then ignored).  fn must not call into
 * this handle. */
typedef int (*spc_observe_fn)(void *user, int64_t step, double t, const double *aos3n);
int spc_run(spc_handle *h, double *t_inout, double dt, int64_t nsteps, int32_t period,
            const uint8_t *observe, spc_observe_fn fn, void *user, int64_t *steps_done);

/* Step counter used as the Philox counter (the number of steps taken). */
int spc_get_step_counter(const spc_handle *h, uint64_t *out);
int spc_set_step_counter(spc_handle *h, uint64_t step);

/* Noise-injection hook: the next steps consume these normals instead of
 * Philox, in the reference's draw order per step (Euler: one per particle,
 * ChimeraSystem.cpp:924-932; SRK: U1 then U2 per particle,
 * StochasticRungeKuttaStepper.hpp:44-45).  count must be a multiple of the
 * per-step count.  Copied to the device; stepping past the end fails with
 * SPC_ERR_NOISE.  spc_clear_noise returns to Philox. */
int spc_inject_noise(spc_handle *h, const double *normals, int64_t count);
int spc_clear_noise(spc_handle *h);
/* Export the Philox normals that steps [first_step, first_step + nsteps)
 * use, in the injection layout, so the same increments can be fed to the
 * reference / oracle. */
int spc_export_noise(spc_handle *h, uint64_t first_step, int32_t nsteps, double *out);
/* Normals per particle per step for this stepper (1, 2 or 0). */
int spc_noise_per_particle(const spc_handle *h);

/* Right-hand sides at the current state, for parity checks.
 * RK form (ChimeraSystem::EvaluateRhs, ChimeraSystem.cpp:78-100): stage
 * state + k_coef*dt*k_prev; k_next (3N, AoS) is read and written: its phase
 * entry is kept where a particle has no neighbour (ChimeraSystem.cpp:421-424). */
int spc_rhs_rk(spc_handle *h, const double *k_prev, double k_coef, double dt, double *k_next);
/* SRK form (ChimeraSystem.cpp:102-114): derivative (3N, AoS) and
 * additional_derivative (2N, [i][0],[i][1]), both zero-started as the
 * steppers do (StochasticRungeKuttaStepper.hpp:36-39). */
int spc_rhs_srk(spc_handle *h, double *derivative, double *additional);

/* Neighbour sets at the current state: counts (n ints) and, if idx is not
 * NULL, the indices of each particle's neighbours concatenated in the
 * reference's visiting order (offsets from the counts).  *total receives the
 * number of pairs; SPC_ERR_CAPACITY if cap is smaller. */
int spc_neighbours(spc_handle *h, int32_t *counts, int32_t *idx, int64_t cap, int64_t *total);

/* Global order parameter R = |<e^{i phi}>| and its argument psi (the
 * observer's summary, BinaryObserver.cpp:196-210, computed in FP64), and the
 * local order parameter mean_i |sum_{j in N_i u {i}} e^{i phi_j}| / (n_i + 1). */
int spc_order_params(spc_handle *h, double *R, double *psi, double *R_local);

/* Diagnostics: clamped cell indices (positions within an ulp of L whose
 * cell index int(x/L*nc) came out as nc), Verlet rebuilds, device error word. */
int spc_diagnostics(spc_handle *h, int64_t *clamped_cells, int64_t *verlet_rebuilds,
                    int64_t *error_word);

/* Per-phase device time of nsteps steps (no graph), measured with CUDA
 * events on the handle's stream between kernel groups.  out_ms receives
 * the average milliseconds per step of: [0] stage + cell keys, [1] radix
 * sort, [2] cell bounds + cell-order gather, [3] first neighbour pass
 * (with its fused epilogue), [4] second neighbour pass (SRK) or the other
 * RK4 passes, [5] the whole step.  On a Verlet handle [0] is the refresh of
 * the Verlet-order state (with the displacement test), [1] the cell binning
 * and [2] the row build, both of which return at once unless the rows must be
 * rebuilt.  cap is out_ms's length (>= 6). */
int spc_profile_steps(spc_handle *h, double dt, int32_t nsteps, double *out_ms, int32_t cap);

/* Tuning knobs (no counterpart in the reference; results do not depend on
 * them beyond floating-point summation order in the FP32C form).
 * SPC_TUNE_SPARSE_BELOW: cell-list systems with fewer particles per cell
 * than this value (on average) run the warp-per-cell neighbour passes, the
 * others the cell-tile passes; 0 sends every system to the cell-tile passes.
 * Default 24.
 * SPC_TUNE_VERLET_ROW_LIMIT (Verlet handles only): the longest neighbour row
 * kept; a particle with more candidates within rho + skin scans its whole
 * cell stencil instead (same results).  Between 1 and the row capacity the
 * handle allocated (its default value); the rows are rebuilt on the next step.
 * SPC_TUNE_TILE_SPLIT: CTAs per cell of the cell-tile passes, 1 to 8, or 0
 * for the default, 1.  Each CTA takes whole groups of the cell's particles
 * (128 in the float forms, 64 in FP64), so a cell of at most one group stays
 * on one CTA and only cells that hold several groups (a clustered state) are
 * spread out.  spc_get_tuning returns the split in effect.  Results are
 * bitwise independent of it in every precision.
 * SPC_TUNE_CELL_UNITS (FP32C and FP32X handles): 1 runs the cells of the
 * cell-tile passes as units of 32 particles x one staging round of their
 * candidate list (cells of more than 8 staging rounds stay whole particle
 * groups), each unit on its own CTA in a second launch of each pass, beside
 * the cell-tile kernel; 0 (the default) runs every cell as whole particle
 * groups.  It pays on clustered states, where whole groups leave most SMs
 * idle at the end of a pass.  With 1, FP32X results are unchanged (exact
 * sums) and FP32C sums are added in another fixed order; either way they do
 * not depend on SPC_TUNE_TILE_SPLIT.  Refused for FP64 handles.
 * SPC_TUNE_SUBCELLS (FP32C and FP32X cell-list handles; the cell-size
 * dimension): 1 bins each cell of side L/int(L/rho) into a lower and an
 * upper half and runs the cells of at most 8 staging rounds as cell units of
 * their halves (with SPC_TUNE_CELL_UNITS 0 as well).  A half needs only the
 * near half of the row beyond it: the far half is more than a cell side
 * (>= rho) away, so about 7.5 of the 9 stencil cells are tested.  0 (the
 * default) keeps whole cells.  The neighbour sets are those of whole cells:
 * FP32X results are unchanged, FP32C sums are added in another fixed
 * order.  (An excluded pair could only count as a neighbour if the cell side
 * equalled rho to within rounding and the pair lay within rounding of the
 * cutoff, across the half boundary, with |dx| below ~1e-8 rho.)  Neighbour
 * diagnostics keep whole cells.  Refused for FP64 and Verlet handles.
 * spc_get_tuning reads a knob back. */
enum {
  SPC_TUNE_SPARSE_BELOW = 1,
  SPC_TUNE_VERLET_ROW_LIMIT = 2,
  SPC_TUNE_TILE_SPLIT = 3,
  SPC_TUNE_CELL_UNITS = 4,
  SPC_TUNE_SUBCELLS = 5
};
int spc_set_tuning(spc_handle *h, int32_t key, double value);
int spc_get_tuning(const spc_handle *h, int32_t key, double *value);

/* Autotuner (no counterpart in the reference).  Times `trial_steps` steps
 * (as captured graphs, after one warm-up call) of every candidate on the
 * caller's state and keeps the fastest: the cell-list passes with the
 * cell-tile or the warp-per-cell kernels, and, where the stencil allows
 * Verlet rows, rows with skins of 0.1, 0.2 and 0.4 rho.  Every candidate
 * computes the same neighbour sets; FP64 results differ between them only by
 * summation order.  omega is required for the vortex model.  On return *best
 * holds p with the winning neighbour method and skin, *sparse_below the
 * SPC_TUNE_SPARSE_BELOW value to set on the handle, and (when not NULL)
 * ms_out[k] the milliseconds per step of candidate k for k < min(cap, count),
 * *count the number of candidates.  The caller's state is not touched. */
/* One tuning candidate and its measured cost (no counterpart in the
 * reference): the neighbour method and skin, the SPC_TUNE_SPARSE_BELOW,
 * SPC_TUNE_TILE_SPLIT, SPC_TUNE_CELL_UNITS and SPC_TUNE_SUBCELLS values, and
 * milliseconds per step. */
typedef struct spc_tuning {
  int32_t neighbour;    /* SPC_NEIGHBOUR_* */
  int32_t tile_split;   /* CTAs per cell of the cell-tile passes */
  double skin;          /* Verlet skin (0 for the cell list) */
  double sparse_below;  /* SPC_TUNE_SPARSE_BELOW value */
  double ms_per_step;   /* measured */
  int32_t cell_units;  /* SPC_TUNE_CELL_UNITS value */
  int32_t subcells;    /* SPC_TUNE_SUBCELLS value */
} spc_tuning;

/* Autotuner over every tuning dimension (no counterpart in the reference):
 * the cell-list passes with each kernel choice (all cell-tile, the default
 * split between cell-tile and warp-per-cell, all warp-per-cell) and, for the
 * cell-tile kernels, 1, 2 or 4 CTAs per cell; and Verlet rows with skins of
 * 0.1, 0.2 and 0.4 rho where the stencil and the precision allow.  Each
 * candidate runs trial_steps steps as a captured graph on its own handle
 * (after a warm-up call) from the caller's state, which is not touched.
 * cands[k] (k < cap) receives candidate k with its cost, *count the number of
 * candidates, *best the fastest's index.  Every candidate computes the same
 * neighbour sets; FP64 and FP32X results are bitwise the same across the
 * kernel choices, FP64 Verlet rows differ from the cell list by summation
 * order, FP32C results by float rounding. */
int spc_autotune_ex(const spc_params *p, int32_t n, const double *aos3n, const double *omega, double dt,
                    int32_t trial_steps, spc_tuning *cands, int32_t cap, int32_t *count, int32_t *best);

/* In-place retuning of a running handle (no counterpart in the reference):
 * as the state evolves (a clustering system's cells fill up) the best kernel
 * choice can change.  Times trial_steps steps of each kernel-choice
 * candidate of spc_autotune_ex (not the neighbour method) on the current
 * state, putting the state, RK4 rates and step counters back after every
 * trial, and keeps the fastest setting.  The state and counters on return
 * are those on entry.  Uses Philox noise (SPC_ERR_STATE while injected noise
 * is pending); allocates a temporary copy of the pool state; synchronises. */
int spc_retune(spc_handle *h, double dt, int32_t trial_steps, spc_tuning *cands, int32_t cap, int32_t *count,
               int32_t *best);

int spc_autotune(const spc_params *p, int32_t n, const double *aos3n, const double *omega, double dt,
                 int32_t trial_steps, spc_params *best, double *sparse_below, double *ms_out,
                 int32_t cap, int32_t *count);

/* Nodes (kernel launches) of the CUDA graph the last spc_step_graph call
 * captured or replayed: every replay launches exactly this many kernels. */
int spc_graph_nodes(const spc_handle *h, int64_t *nodes);
/* Nodes of spc_run's captured chunk graph (0 if none) and its steps. */
int spc_run_graph_nodes(const spc_handle *h, int64_t *nodes, int32_t *steps);

/* Synchronise the handle's stream; the stream itself (a cudaStream_t) for
 * callers that time or order work around the library. */
int spc_synchronize(spc_handle *h);
void *spc_stream(spc_handle *h);

/* Philox4x32-10 evaluated on the device (the generator behind every noise
 * draw), for checking against the published known-answer vectors. */
int spc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Self-check of the FP64 kernels' division by a reused divisor (no reference
 * counterpart): for i < n, a[i] / b[i] on the device both as the correctly
 * rounded division and as the kernels' form (reciprocal rounded to nearest,
 * then one fused multiply-add correction); *mismatches counts the pairs
 * whose results differ in any bit (0 means the FP64 forms divide exactly as
 * the reference writes it). */
int spc_check_division(int64_t n, const double *a, const double *b, int64_t *mismatches);

/* Self-check of the FP64 Verlet passes' cosine cache (no reference
 * counterpart): for i < n, sin(x[i]) and cos(x[i]) from separate launches
 * against one sincos(x[i]); *mismatches counts the values whose results
 * differ in any bit (0 means the cached cosine of the first pass is the
 * cosine the second pass would compute). */
int spc_check_sincos(int64_t n, const double *x, int64_t *mismatches);

/* ---------------------------------------------------------------------------
 * Batches: many independent systems (each with its own N, box and
 * parameters) resident in one pool of device memory and advanced together,
 * one kernel launch per phase for all of them.  The reference runs one system
 * per process (its parameter scan gives each MPI rank one system,
 * main.cpp:15-18); here a batch replaces that, and a serving loop admits and
 * releases systems between calls.  All systems of a batch share the stepper
 * and precision; dt is per call.  A system admitted with a step budget is
 * frozen once it has taken that many steps (later steps leave it unchanged),
 * so requests of different lengths finish exactly.  A system's trajectory is
 * the same alone or in a batch: its noise is keyed by (seed, system_id,
 * step, particle) and its neighbour sums never see another system.
 * ------------------------------------------------------------------------- */
typedef struct spc_batch spc_batch;

typedef struct spc_batch_config {
  int32_t stepper;       /* SPC_STEPPER_* of every system */
  int32_t precision;     /* SPC_PRECISION_* of every system */
  int32_t max_systems;   /* system slots */
  int32_t pad;
  int64_t max_particles; /* pool capacity (sum of N) */
  int64_t max_cells;     /* sum over systems of int(L/rho)^2 (1 per all-pairs system) */
} spc_batch_config;

/* Device bytes a batch reserves per pool particle and per cell, for
 * admission control by memory footprint. */
int spc_batch_footprint(int32_t stepper, int32_t precision, int64_t *bytes_per_particle,
                        int64_t *bytes_per_cell);
int spc_batch_create(const spc_batch_config *cfg, spc_batch **out);
int spc_batch_destroy(spc_batch *b);
const char *spc_batch_last_error(const spc_batch *b);
/* Admit a system (the engine's ctor + state upload, SimulationEngine.cpp:31-50):
 * aos3n is its initial state, omega its natural frequencies (vortex model,
 * else NULL), steps its step budget (-1: unlimited).  SPC_ERR_CAPACITY when
 * the pool has no contiguous room for n particles, or no free cells or slot. */
int spc_batch_admit(spc_batch *b, const spc_params *p, int32_t n, const double *aos3n,
                    const double *omega, int64_t steps, int32_t *slot);
int spc_batch_release(spc_batch *b, int32_t slot);
/* nsteps steps of every admitted system (DoStep + wrap each, as spc_step). */
int spc_batch_step(spc_batch *b, double dt, int32_t nsteps);
int spc_batch_step_graph(spc_batch *b, double dt, int32_t nsteps);
int spc_batch_download(spc_batch *b, int32_t slot, double *aos3n);
int spc_batch_upload(spc_batch *b, int32_t slot, const double *aos3n);
int spc_batch_status(spc_batch *b, int32_t slot, uint64_t *steps_done, int64_t *remaining);
int spc_batch_usage(spc_batch *b, int64_t *particles, int64_t *cells, int32_t *systems);
int spc_batch_order_params(spc_batch *b, int32_t slot, double *R, double *psi);
/* Order parameters of every system of the batch in one call (the per-frame
 * summary of BinaryObserver.cpp:196-210 for each system, plus the local order
 * parameter of spc_order_params): entry s of R, psi and R_local (each may be
 * NULL) is slot s's, for s < cap; slots without a system get NaN.  One
 * diagnostics pass over the whole batch; synchronises the batch's stream. */
int spc_batch_order_params_all(spc_batch *b, int32_t cap, double *R, double *psi, double *R_local);
int spc_batch_synchronize(spc_batch *b);
void *spc_batch_stream(spc_batch *b);
/* Per-phase device time of nsteps steps of the whole batch (as
 * spc_profile_steps; the steps count against the systems' budgets). */
int spc_batch_profile_steps(spc_batch *b, double dt, int32_t nsteps, double *out_ms, int32_t cap);
/* The tuning knobs of spc_set_tuning, for a whole batch. */
int spc_batch_set_tuning(spc_batch *b, int32_t key, double value);
int spc_batch_get_tuning(const spc_batch *b, int32_t key, double *value);
/* spc_retune for a whole batch: the kernel choice of every system at once. */
int spc_batch_retune(spc_batch *b, double dt, int32_t trial_steps, spc_tuning *cands, int32_t cap,
                     int32_t *count, int32_t *best);

/* SRK-form right-hand side (as spc_rhs_srk) computed without allocating
 * any device memory.  No counterpart in the reference: it exists for callers
 * that must not call cudaMalloc, such as code whose device memory is owned by
 * another component's pool, latency-critical loops where an allocation would
 * synchronise the device, or processes that fix their device footprint at
 * start-up.  The caller passes device buffers: d_state (3N doubles, AoS),
 * d_derivative (3N) and d_additional (2N); the work is enqueued on `stream`
 * (a cudaStream_t, NULL for the default stream) and the call returns without
 * waiting.  Intermediates live in one static device array of about 1.1 MB
 * that every GPU loading the library keeps until the process exits; limits:
 * n <= 8192 particles and int(L/rho)^2 <= 16384 cells, larger sizes return
 * SPC_ERR_CAPACITY.  The Chimera and vortex models are supported; the
 * vortex-arrays model returns SPC_ERR_INVALID.  Positions in d_state must
 * already be wrapped into [0, L), as after any step: the call does not wrap
 * them, and cell indices of positions outside are clamped without a report.
 * The first call on a device looks up that array's device address (with the
 * device current) and caches it with the current context; a call in another
 * context, e.g. after cudaDeviceReset, looks it up again.  So make the first
 * call, and the first after a reset, before any stream capture.  All calls
 * share the one array: calls whose work overlaps on the GPU (different
 * streams, or different host threads) race and must be ordered by the
 * caller. */
int spc_rhs_srk_noalloc(const spc_params *p, int32_t n, const double *d_state,
                        double *d_derivative, double *d_additional, void *stream);

/* Page-locked host buffers for callers that stream state in and out. */
int spc_alloc_pinned(size_t bytes, void **out);
int spc_free_pinned(void *p);

#ifdef __cplusplus
}
#endif
#endif
