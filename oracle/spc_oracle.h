/*
 * spc_oracle.h -- CPU restatement of the particle-update path of
 * raven91/spc2_langevin_integration (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  The product path (the CUDA library behind
 * include/spc_gb300.h) never links, loads or calls this code; only the test
 * suite, the smoke check and the CPU-baseline leg of bench.py use it, and only
 * as the checker / the timed CPU reference.
 *
 * Every routine restates one reference routine in plain C with the same
 * floating-point operation order (compiled with -ffp-contract=off so that no
 * multiply-add is fused), so that on identical inputs and identical injected
 * normals it reproduces the reference's FP64 results.  The restatement is
 * pinned against the reference itself: oracle/ref builds the reference's own
 * sources (unmodified) into oracle/_ref, and tests/golden holds vectors made
 * with it.
 *
 * State layout follows the reference: array-of-structures [x0,y0,phi0,x1,...]
 * of length 3N (Definitions.hpp:21 kS = 3).
 */
#ifndef SPC_ORACLE_H
#define SPC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_EULER = 0, ORC_SRK = 1, ORC_RK4 = 2, ORC_EULER_PTR = 3 };

typedef struct orc_system orc_system;

/* ChimeraSystem ctor (DynamicalSystems/ChimeraSystem.cpp:11-59) together with
 * the PeriodicBoundaryConditions it holds (PeriodicBoundaryConditions.cpp:7-17).
 * Returns NULL on a bad argument (n <= 0, L <= 0, rho <= 0). */
orc_system *orc_create(int n, double L, double v0, double sigma, double rho,
                       double alpha, double D_phi);
void orc_destroy(orc_system *s);

/* Number of cells per side, int(L / rho) (ChimeraSystem.cpp:32-33). */
int orc_num_cells(const orc_system *s);
/* 1 when EvaluateRhs takes the cell-list path (rho <= 0.25 L,
 * ChimeraSystem.cpp:90), 0 for the all-pairs path. */
int orc_uses_cell_list(const orc_system *s);
/* Particles whose cell index fell outside [0, nc) and were clamped (the
 * reference indexes out of bounds there); cumulative. */
long long orc_clamped_cells(const orc_system *s);

/* ClassAEffectiveParticleDistance (PeriodicBoundaryConditions.cpp:22-35). */
void orc_min_image(const orc_system *s, double xi, double yi, double xj,
                   double yj, double *dx, double *dy);
/* ApplyPeriodicBoundaryConditions scalar form (:117-121). */
void orc_wrap_point(const orc_system *s, double x, double y, double *xp,
                    double *yp);
/* Engine-level wrap of the whole state (:123-131), x and y only. */
void orc_wrap_state(const orc_system *s, double *state);

/* RK-form EvaluateRhs (ChimeraSystem.cpp:78-100 -> :117-168 / :258-426).
 * k_prev may alias k_next.  counts (may be NULL) receives n_i per particle. */
void orc_rhs_rk(orc_system *s, const double *state, const double *k_prev,
                double *k_next, double k_coef, double dt, int *counts);
/* SRK-form EvaluateRhs (ChimeraSystem.cpp:102-114 -> :171-255 / :429-645).
 * derivative (3N) and additional (2N, [i][0], [i][1]) are accumulated into as
 * in the reference; callers zero them first, as the steppers do. */
void orc_rhs_srk(orc_system *s, const double *state, double *derivative,
                 double *additional, int *counts);

/* Steppers.  noise holds the normals of one step in the reference's draw
 * order: Euler one per particle (ChimeraSystem.cpp:924-932), SRK U1 then U2
 * per particle (StochasticRungeKuttaStepper.hpp:44-45).  omega (may be NULL)
 * are the natural frequencies of StochasticRungeKuttaStepperPtr (:65); the
 * Euler stepper, which has no frequency form in the reference, adds them to
 * its phase drift the same way (an extension for vortex systems). */
void orc_step_euler(orc_system *s, double *state, double t, double dt,
                    const double *noise, const double *omega);
void orc_step_euler_ptr(orc_system *s, double *state, double t, double dt,
                        const double *noise);
void orc_step_srk(orc_system *s, double *state, double t, double dt,
                  const double *noise, const double *omega);
void orc_step_rk4(orc_system *s, double *state, double t, double dt);

/* Engine loop (SimulationEngine.cpp:149-161): t += dt; DoStep; wrap.  noise
 * holds nsteps consecutive per-step blocks (N or 2N normals each, none for
 * RK4).  Returns the final t. */
double orc_run(orc_system *s, int stepper, double *state, double t0, double dt,
               int nsteps, const double *noise, const double *omega);

/* The RK4 stage buffers k1..k4 persist across steps (RungeKutta4Stepper.cpp:7-13);
 * read/write them for resume and tests (4 x 3N doubles). */
void orc_get_rk4_buffers(const orc_system *s, double *out);
void orc_set_rk4_buffers(orc_system *s, const double *in);

/* Neighbour lists of the cell-list (or all-pairs) search at the given stage
 * positions: for particle i, indices[offsets[i] .. offsets[i+1]) in the
 * reference's visiting order.  offsets has N+1 entries; indices capacity is
 * cap.  Returns the total count (which may exceed cap; then nothing past cap
 * is written). */
long long orc_neighbour_lists(orc_system *s, const double *stage_state,
                              long long *offsets, int *indices, long long cap);

/* Order parameters of the phases: global R = |mean e^{i phi}| and its
 * argument in FP64, the reference observer's float form
 * (BinaryObserver.cpp:196-210), and the local order parameter
 * mean_i |sum_{j in N_i u {i}} e^{i phi_j}| / (n_i + 1) over the cell-list
 * neighbourhoods at the given state. */
void orc_order_params(orc_system *s, const double *state, double *R,
                      double *psi, float *R_f32, float *psi_f32,
                      double *R_local);

/* VortexArraysSystemPtr (DynamicalSystems/VortexArraysSystemPtr.cpp): the
 * reference's second model, alignment mu+ / anti-alignment mu- by distance and
 * cohesion kappa (ctor :9-88; RHS :357-507 RK form, :509-735 SRK form, all
 * pairs :136-355).  Destroy with orc_destroy; the RK4 buffers are
 * orc_get/set_rk4_buffers.  counts3 (may be NULL) receives per particle the
 * three neighborhood_cardinality_ entries. */
orc_system *orc_va_create(int n, double L, double velocity, double mu_plus, double mu_minus,
                          double xi_a, double xi_r, double D_phi, double kappa, double rho);
void orc_va_rhs_rk(orc_system *s, const double *state, const double *k_prev, double *k_next,
                   double k_coef, double dt, int *counts3);
void orc_va_rhs_srk(orc_system *s, const double *state, double *derivative, double *additional,
                    int *counts3);
/* Engine loop with StochasticEulerStepperPtr (ORC_EULER_PTR, N normals per
 * step), StochasticRungeKuttaStepperPtr (ORC_SRK, 2N: U1, U2 per particle) or
 * RungeKutta4StepperPtr (ORC_RK4, no noise). */
double orc_va_run(orc_system *s, int stepper, double *state, double t0, double dt, int nsteps,
                  const double *noise);

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds on counter
 * ctr[4] with key key[2]; out[4]. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
