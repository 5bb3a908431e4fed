/*
 * spc_oracle.c -- CPU restatement of the reference's particle-update path.
 *
 * TEST INFRASTRUCTURE ONLY (see spc_oracle.h): used by tests/, the smoke check
 * and bench.py's CPU-baseline leg as the checker; never by the product path.
 *
 * Build with -O2 -ffp-contract=off (oracle/build_oracle.py does): every
 * expression below keeps the reference's evaluation order, and no product may
 * be fused into an add, so the FP64 results equal the reference's bit for bit
 * on the same libm.  Citations are file:line in raven91/spc2_langevin_integration.
 */
#include "spc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct orc_system {
  int n;
  double L, rL; /* x_size_, x_rsize_ = 1.0 / x_size (PeriodicBoundaryConditions.cpp:13-14) */
  double v0, sigma, rho, rho2, alpha, D_phi;
  int nc;       /* num_subcells_ = int(kL / rho) (ChimeraSystem.cpp:32-33) */
  long long clamped;
  /* scratch */
  double *rk;       /* stage state, the function-static rk_system_state (:270) */
  double *af, *card;/* alignment_force_, neighborhood_cardinality_ (:28-29) */
  int *key;         /* pre_linked_list_ (:35) */
  int *cell_start;  /* linked_list_ as CSR: cells hold ascending indices (:335-338) */
  int *cell_fill;
  int *cell_items;
  double *det, *sto;    /* StochasticEulerStepper statics (StochasticEulerStepper.hpp:33) */
  double *deriv, *addl; /* StochasticRungeKuttaStepper statics (StochasticRungeKuttaStepper.hpp:36-38) */
  double *k[4];         /* RungeKutta4Stepper members (RungeKutta4Stepper.cpp:7-13) */
  /* VortexArraysSystemPtr (VortexArraysSystemPtr.cpp:9-38); v0 is velocity_ */
  int va;
  double mu_plus, mu_minus, xi_a, xi_r, kappa;
  double *anti, *coh;   /* antialignment_force_, cohesion_force_ */
  double *card1, *card2;/* neighborhood_cardinality_[i][1], [i][2] ([i][0] is card) */
};

/* neighboring_cells_ in visiting order, {dx, dy} (ChimeraSystem.cpp:39-44) */
static const int kStencil[9][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {0, 0},
                                   {1, 0},   {-1, 1}, {0, 1},  {1, 1}};

orc_system *orc_create(int n, double L, double v0, double sigma, double rho,
                       double alpha, double D_phi) {
  if (n <= 0 || !(L > 0.0) || !(rho > 0.0)) return NULL;
  orc_system *s = (orc_system *)calloc(1, sizeof(orc_system));
  if (!s) return NULL;
  s->n = n;
  s->L = L;
  s->rL = 1.0 / L;
  s->v0 = v0;
  s->sigma = sigma;
  s->rho = rho;
  s->rho2 = rho * rho; /* rho_squared_ (ChimeraSystem.cpp:24) */
  s->alpha = alpha;
  s->D_phi = D_phi;
  s->nc = (int)(L / rho);
  if (s->nc < 1) s->nc = 1;
  size_t n3 = (size_t)3 * (size_t)n;
  size_t ncell = (size_t)s->nc * (size_t)s->nc;
  s->rk = (double *)calloc(n3, sizeof(double));
  s->af = (double *)calloc((size_t)n, sizeof(double));
  s->card = (double *)calloc((size_t)n, sizeof(double));
  s->key = (int *)calloc((size_t)n, sizeof(int));
  s->cell_start = (int *)calloc(ncell + 1, sizeof(int));
  s->cell_fill = (int *)calloc(ncell, sizeof(int));
  s->cell_items = (int *)calloc((size_t)n, sizeof(int));
  s->det = (double *)calloc(n3, sizeof(double));
  s->sto = (double *)calloc(n3, sizeof(double));
  s->deriv = (double *)calloc(n3, sizeof(double));
  s->addl = (double *)calloc((size_t)2 * (size_t)n, sizeof(double));
  for (int q = 0; q < 4; ++q) s->k[q] = (double *)calloc(n3, sizeof(double));
  if (!s->rk || !s->af || !s->card || !s->key || !s->cell_start ||
      !s->cell_fill || !s->cell_items || !s->det || !s->sto || !s->deriv ||
      !s->addl || !s->k[0] || !s->k[1] || !s->k[2] || !s->k[3]) {
    orc_destroy(s);
    return NULL;
  }
  return s;
}

void orc_destroy(orc_system *s) {
  if (!s) return;
  free(s->rk);
  free(s->af);
  free(s->card);
  free(s->key);
  free(s->cell_start);
  free(s->cell_fill);
  free(s->cell_items);
  free(s->det);
  free(s->sto);
  free(s->deriv);
  free(s->addl);
  for (int q = 0; q < 4; ++q) free(s->k[q]);
  free(s->anti);
  free(s->coh);
  free(s->card1);
  free(s->card2);
  free(s);
}

int orc_num_cells(const orc_system *s) { return s->nc; }
int orc_uses_cell_list(const orc_system *s) { return s->rho <= 0.25 * s->L; }
long long orc_clamped_cells(const orc_system *s) { return s->clamped; }

/* PeriodicBoundaryConditions.cpp:22-35 */
void orc_min_image(const orc_system *s, double xi, double yi, double xj,
                   double yj, double *dx, double *dy) {
  double ddx = xj - xi;
  ddx -= (double)(int)(ddx * 2.0 * s->rL) * s->L;
  double ddy = yj - yi;
  ddy -= (double)(int)(ddy * 2.0 * s->rL) * s->L;
  *dx = ddx;
  *dy = ddy;
}

/* PeriodicBoundaryConditions.cpp:117-121 */
void orc_wrap_point(const orc_system *s, double x, double y, double *xp,
                    double *yp) {
  *xp = x - floor(x * s->rL) * s->L;
  *yp = y - floor(y * s->rL) * s->L;
}

/* PeriodicBoundaryConditions.cpp:123-131 */
void orc_wrap_state(const orc_system *s, double *state) {
  for (int i = 0; i < s->n; ++i) {
    state[3 * i] -= floor(state[3 * i] * s->rL) * s->L;
    state[3 * i + 1] -= floor(state[3 * i + 1] * s->rL) * s->L;
  }
}

/* Conditional wrap applied to copies inside the force loops
 * (ChimeraSystem.cpp:299-302, :373-376, :402-405). */
static inline void wrap_if_outside(const orc_system *s, double *x, double *y) {
  if (*x < 0.0 || *x >= s->L || *y < 0.0 || *y >= s->L) {
    double xw = *x - floor(*x * s->rL) * s->L;
    double yw = *y - floor(*y * s->rL) * s->L;
    *x = xw;
    *y = yw;
  }
}

/* i_cell_x = int(x / x_size_ * num_subcells_x_) (ChimeraSystem.cpp:304-306).
 * An index outside [0, nc) (x within an ulp of L, hazard "H3") is clamped
 * here; the reference would index out of bounds. */
static inline int cell_coord(orc_system *s, double x, int count) {
  int c = (int)(x / s->L * (double)s->nc);
  if (c < 0 || c >= s->nc) {
    c = c < 0 ? 0 : s->nc - 1;
    if (count) s->clamped++;
  }
  return c;
}

/* AdjustNeighboringCellToPeriodicBoundaries (ChimeraSystem.cpp:905-922) */
static inline int adjust_cell(int c, int nc) {
  if (c < 0) return nc - 1;
  if (c >= nc) return 0;
  return c;
}

/* Cell binning of positions pos (3N, AoS) into the CSR linked list
 * (ChimeraSystem.cpp:279-338). */
static void build_linked_list(orc_system *s, const double *pos) {
  const int n = s->n, nc = s->nc;
  const size_t ncell = (size_t)nc * (size_t)nc;
  for (int i = 0; i < n; ++i) {
    double x = pos[3 * i], y = pos[3 * i + 1];
    wrap_if_outside(s, &x, &y);
    int cx = cell_coord(s, x, 1);
    int cy = cell_coord(s, y, 1);
    s->key[i] = cy * nc + cx;
  }
  memset(s->cell_start, 0, (ncell + 1) * sizeof(int));
  for (int i = 0; i < n; ++i) s->cell_start[s->key[i] + 1]++;
  for (size_t c = 0; c < ncell; ++c) s->cell_start[c + 1] += s->cell_start[c];
  memset(s->cell_fill, 0, ncell * sizeof(int));
  for (int i = 0; i < n; ++i) {
    int c = s->key[i];
    s->cell_items[s->cell_start[c] + s->cell_fill[c]++] = i;
  }
}

/* Visit the cell-list neighbours j of i (j != i, dr^2 <= rho^2) in the
 * reference's order: stencil order, ascending index within a cell
 * (ChimeraSystem.cpp:365-418).  pos must be the binned positions. */
typedef void (*visit_fn)(void *ctx, int i, int j, const double *pos);

static void for_each_cell_neighbour(orc_system *s, const double *pos, int i,
                                    visit_fn fn, void *ctx) {
  const int nc = s->nc;
  double xi = pos[3 * i], yi = pos[3 * i + 1];
  wrap_if_outside(s, &xi, &yi);
  int cx = cell_coord(s, xi, 0);
  int cy = cell_coord(s, yi, 0);
  for (int q = 0; q < 9; ++q) {
    int jx = adjust_cell(cx + kStencil[q][0], nc);
    int jy = adjust_cell(cy + kStencil[q][1], nc);
    int c = jy * nc + jx;
    for (int p = s->cell_start[c]; p < s->cell_start[c + 1]; ++p) {
      int j = s->cell_items[p];
      if (j == i) continue;
      double xj = pos[3 * j], yj = pos[3 * j + 1];
      wrap_if_outside(s, &xj, &yj);
      double dx, dy;
      orc_min_image(s, xi, yi, xj, yj, &dx, &dy);
      double dr2 = dx * dx + dy * dy;
      if (dr2 <= s->rho2) fn(ctx, i, j, pos);
    }
  }
}

/* All-pairs neighbours (ChimeraSystem.cpp:139-159): positions are NOT wrapped
 * before the minimum-image distance. */
static void for_each_allpairs_neighbour(orc_system *s, const double *pos, int i,
                                        visit_fn fn, void *ctx) {
  const double xi = pos[3 * i], yi = pos[3 * i + 1];
  for (int j = 0; j < s->n; ++j) {
    if (j == i) continue;
    double dx, dy;
    orc_min_image(s, xi, yi, pos[3 * j], pos[3 * j + 1], &dx, &dy);
    double dr2 = dx * dx + dy * dy;
    if (dr2 <= s->rho2) fn(ctx, i, j, pos);
  }
}

static void for_each_neighbour(orc_system *s, const double *pos, int i,
                               visit_fn fn, void *ctx) {
  if (orc_uses_cell_list(s))
    for_each_cell_neighbour(s, pos, i, fn, ctx);
  else
    for_each_allpairs_neighbour(s, pos, i, fn, ctx);
}

/* pass 1 visitor: alignment_force_[i] += sin(phi_j - phi_i - alpha_);
 * ++neighborhood_cardinality_[i] (ChimeraSystem.cpp:410-414) */
static void visit_pass1(void *ctx, int i, int j, const double *pos) {
  orc_system *s = (orc_system *)ctx;
  const double phi_i = pos[3 * i + 2], phi_j = pos[3 * j + 2];
  s->af[i] += sin(phi_j - phi_i - s->alpha);
  s->card[i] += 1.0;
}

typedef struct {
  orc_system *s;
  const double *deriv;
  double *addl;
} pass2_ctx;

/* pass 2 visitor (ChimeraSystem.cpp:632-638) */
static void visit_pass2(void *vctx, int i, int j, const double *pos) {
  pass2_ctx *c = (pass2_ctx *)vctx;
  orc_system *s = c->s;
  if (s->card[i] == 0.0) return;
  const double phi_i = pos[3 * i + 2], phi_j = pos[3 * j + 2];
  c->addl[2 * i] += cos(phi_j - phi_i - s->alpha) / s->card[i];
  c->addl[2 * i + 1] += (c->deriv[3 * j + 2] - c->deriv[3 * i + 2]) *
                        cos(phi_j - phi_i - s->alpha) / s->card[i];
}

void orc_rhs_rk(orc_system *s, const double *state, const double *k_prev,
                double *k_next, double k_coef, double dt, int *counts) {
  const int n = s->n;
  memset(s->af, 0, (size_t)n * sizeof(double));
  memset(s->card, 0, (size_t)n * sizeof(double));
  /* stage state rk = s + k_coef * dt * k_prev (ChimeraSystem.cpp:270-277,
   * :135-137, :146-148); computed for every particle before k_next is
   * written, so k_prev may alias k_next. */
  for (int i = 0; i < 3 * n; ++i) s->rk[i] = state[i] + k_coef * dt * k_prev[i];
  if (orc_uses_cell_list(s)) build_linked_list(s, s->rk);
  for (int i = 0; i < n; ++i) {
    for_each_neighbour(s, s->rk, i, visit_pass1, s);
    const double phi_i = s->rk[3 * i + 2];
    /* ChimeraSystem.cpp:419-424: the phase rate is only written when the
     * particle has neighbours; otherwise k_next keeps its previous value. */
    k_next[3 * i] = s->v0 * cos(phi_i);
    k_next[3 * i + 1] = s->v0 * sin(phi_i);
    if (s->card[i] != 0.0) k_next[3 * i + 2] = s->sigma * s->af[i] / s->card[i];
    if (counts) counts[i] = (int)s->card[i];
  }
}

void orc_rhs_srk(orc_system *s, const double *state, double *derivative,
                 double *additional, int *counts) {
  const int n = s->n;
  memset(s->af, 0, (size_t)n * sizeof(double));
  memset(s->card, 0, (size_t)n * sizeof(double));
  if (orc_uses_cell_list(s)) build_linked_list(s, state);
  /* pass 1 (ChimeraSystem.cpp:526-586) */
  for (int i = 0; i < n; ++i) {
    for_each_neighbour(s, state, i, visit_pass1, s);
    const double phi_i = state[3 * i + 2];
    derivative[3 * i] = s->v0 * cos(phi_i);
    derivative[3 * i + 1] = s->v0 * sin(phi_i);
    if (s->card[i] != 0.0)
      derivative[3 * i + 2] = s->sigma * s->af[i] / s->card[i];
    if (counts) counts[i] = (int)s->card[i];
  }
  /* pass 2 (ChimeraSystem.cpp:589-644) */
  pass2_ctx c = {s, derivative, additional};
  for (int i = 0; i < n; ++i) {
    for_each_neighbour(s, state, i, visit_pass2, &c);
    additional[2 * i] *= -sqrt(2.0 * s->D_phi);
    additional[2 * i + 1] += -2.0 * s->D_phi * derivative[3 * i + 2];
  }
}

/* StochasticEulerStepper::DoStep (StochasticEulerStepper.hpp:31-47) with
 * ChimeraSystem::AddNoise (ChimeraSystem.cpp:924-932). */
void orc_step_euler(orc_system *s, double *state, double t, double dt,
                    const double *noise, const double *omega) {
  (void)t;
  const int n = s->n;
  memset(s->det, 0, (size_t)3 * n * sizeof(double));
  memset(s->sto, 0, (size_t)3 * n * sizeof(double));
  orc_rhs_rk(s, state, s->det, s->det, 0.0, dt, NULL);
  const double intensity = sqrt(2.0 * s->D_phi);
  for (int i = 0; i < n; ++i) s->sto[3 * i + 2] = intensity * noise[i];
  for (int i = 0; i < n; ++i) {
    state[3 * i] += dt * s->det[3 * i] + sqrt(dt) * s->sto[3 * i];
    state[3 * i + 1] += dt * s->det[3 * i + 1] + sqrt(dt) * s->sto[3 * i + 1];
    if (omega) /* frequencies in the drift, as StochasticRungeKuttaStepperPtr.hpp:65 */
      state[3 * i + 2] += dt * (omega[i] + s->det[3 * i + 2]) + sqrt(dt) * s->sto[3 * i + 2];
    else
      state[3 * i + 2] += dt * s->det[3 * i + 2] + sqrt(dt) * s->sto[3 * i + 2];
  }
}

/* StochasticEulerStepperPtr::DoStep (StochasticEulerStepperPtr.hpp:32-53):
 * SRK-form right-hand side (its second pass is unused), then
 * phi += f dt + sqrt(2D) (sqrt(dt) xi). */
void orc_step_euler_ptr(orc_system *s, double *state, double t, double dt,
                        const double *noise) {
  (void)t;
  const int n = s->n;
  memset(s->deriv, 0, (size_t)3 * n * sizeof(double));
  memset(s->addl, 0, (size_t)2 * n * sizeof(double));
  orc_rhs_srk(s, state, s->deriv, s->addl, NULL);
  for (int i = 0; i < n; ++i) {
    double delta_W = sqrt(dt) * noise[i];
    state[3 * i] += s->deriv[3 * i] * dt;
    state[3 * i + 1] += s->deriv[3 * i + 1] * dt;
    state[3 * i + 2] += s->deriv[3 * i + 2] * dt + sqrt(2.0 * s->D_phi) * delta_W;
  }
}

/* StochasticRungeKuttaStepper::DoStep (StochasticRungeKuttaStepper.hpp:34-61);
 * with omega, the StochasticRungeKuttaStepperPtr form whose phase drift adds
 * the natural frequency (StochasticRungeKuttaStepperPtr.hpp:65). */
void orc_step_srk(orc_system *s, double *state, double t, double dt,
                  const double *noise, const double *omega) {
  (void)t;
  const int n = s->n;
  memset(s->deriv, 0, (size_t)3 * n * sizeof(double));
  memset(s->addl, 0, (size_t)2 * n * sizeof(double));
  orc_rhs_srk(s, state, s->deriv, s->addl, NULL);
  const double D = s->D_phi;
  for (int i = 0; i < n; ++i) {
    double U_1 = noise[2 * i], U_2 = noise[2 * i + 1];
    double delta_W = U_1 * sqrt(dt);
    double delta_Z = 0.5 * dt * sqrt(dt) * (U_1 + U_2 / sqrt(3.0));
    const double *d = s->deriv + 3 * i;
    const double *a = s->addl + 2 * i;
    state[3 * i] += d[0] * dt - sqrt(2.0 * D) * d[1] * delta_Z -
                    0.5 * (d[2] * d[1] + D * d[0]) * dt * dt;
    state[3 * i + 1] += d[1] * dt + sqrt(2.0 * D) * d[0] * delta_Z +
                        0.5 * (d[2] * d[0] - D * d[1]) * dt * dt;
    if (omega)
      state[3 * i + 2] += (omega[i] + d[2]) * dt + sqrt(2.0 * D) * delta_W +
                          a[0] * delta_Z + 0.5 * a[1] * dt * dt;
    else
      state[3 * i + 2] += d[2] * dt + sqrt(2.0 * D) * delta_W + a[0] * delta_Z +
                          0.5 * a[1] * dt * dt;
  }
}

/* RungeKutta4Stepper::DoStep (RungeKutta4Stepper.cpp:29-57).  The k buffers
 * persist, so an isolated particle keeps its previous phase rate. */
void orc_step_rk4(orc_system *s, double *state, double t, double dt) {
  (void)t;
  double *k1 = s->k[0], *k2 = s->k[1], *k3 = s->k[2], *k4 = s->k[3];
  orc_rhs_rk(s, state, k1, k1, 0.0, dt, NULL);
  orc_rhs_rk(s, state, k1, k2, 0.5, dt, NULL);
  orc_rhs_rk(s, state, k2, k3, 0.5, dt, NULL);
  orc_rhs_rk(s, state, k3, k4, 1.0, dt, NULL);
  for (int i = 0; i < s->n; ++i) {
    int ii = 3 * i;
    state[ii] += (k1[ii] + 2.0 * k2[ii] + 2.0 * k3[ii] + k4[ii]) * dt / 6.0;
    state[ii + 1] +=
        (k1[ii + 1] + 2.0 * k2[ii + 1] + 2.0 * k3[ii + 1] + k4[ii + 1]) * dt / 6.0;
    state[ii + 2] +=
        (k1[ii + 2] + 2.0 * k2[ii + 2] + 2.0 * k3[ii + 2] + k4[ii + 2]) / 6.0 * dt;
  }
}

double orc_run(orc_system *s, int stepper, double *state, double t0, double dt,
               int nsteps, const double *noise, const double *omega) {
  double t = t0;
  const int n = s->n;
  for (int k = 0; k < nsteps; ++k) {
    t += dt;
    switch (stepper) {
      case ORC_EULER:
        orc_step_euler(s, state, t, dt, noise + (size_t)k * n, omega);
        break;
      case ORC_EULER_PTR:
        orc_step_euler_ptr(s, state, t, dt, noise + (size_t)k * n);
        break;
      case ORC_SRK:
        orc_step_srk(s, state, t, dt, noise + (size_t)k * 2 * n, omega);
        break;
      default:
        orc_step_rk4(s, state, t, dt);
        break;
    }
    orc_wrap_state(s, state); /* SimulationEngine.cpp:154 */
  }
  return t;
}

void orc_get_rk4_buffers(const orc_system *s, double *out) {
  size_t n3 = (size_t)3 * s->n;
  for (int q = 0; q < 4; ++q) memcpy(out + q * n3, s->k[q], n3 * sizeof(double));
}

void orc_set_rk4_buffers(orc_system *s, const double *in) {
  size_t n3 = (size_t)3 * s->n;
  for (int q = 0; q < 4; ++q) memcpy(s->k[q], in + q * n3, n3 * sizeof(double));
}

typedef struct {
  long long pos, cap;
  int *indices;
} list_ctx;

static void visit_collect(void *vctx, int i, int j, const double *p) {
  (void)i;
  (void)p;
  list_ctx *c = (list_ctx *)vctx;
  if (c->pos < c->cap) c->indices[c->pos] = j;
  c->pos++;
}

long long orc_neighbour_lists(orc_system *s, const double *stage_state,
                              long long *offsets, int *indices, long long cap) {
  if (orc_uses_cell_list(s)) build_linked_list(s, stage_state);
  list_ctx c = {0, cap, indices};
  for (int i = 0; i < s->n; ++i) {
    offsets[i] = c.pos;
    for_each_neighbour(s, stage_state, i, visit_collect, &c);
  }
  offsets[s->n] = c.pos;
  return c.pos;
}

typedef struct {
  double re, im;
  int cnt;
} local_ctx;

static void visit_local(void *vctx, int i, int j, const double *pos) {
  (void)i;
  local_ctx *c = (local_ctx *)vctx;
  c->re += cos(pos[3 * j + 2]);
  c->im += sin(pos[3 * j + 2]);
  c->cnt++;
}

void orc_order_params(orc_system *s, const double *state, double *R,
                      double *psi, float *R_f32, float *psi_f32,
                      double *R_local) {
  const int n = s->n;
  double re = 0.0, im = 0.0;
  float fre = 0.0f, fim = 0.0f;
  for (int i = 0; i < n; ++i) {
    double c = cos(state[3 * i + 2]), sn = sin(state[3 * i + 2]);
    re += c;
    im += sn;
    /* BinaryObserver.cpp:204-205: complex<float> of the float-cast cos/sin */
    fre += (float)c;
    fim += (float)sn;
  }
  re /= n;
  im /= n;
  fre /= (float)n;
  fim /= (float)n;
  if (R) *R = hypot(re, im);
  if (psi) *psi = atan2(im, re);
  if (R_f32) *R_f32 = hypotf(fre, fim);
  if (psi_f32) *psi_f32 = atan2f(fim, fre);
  if (R_local) {
    if (orc_uses_cell_list(s)) build_linked_list(s, state);
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
      local_ctx c = {cos(state[3 * i + 2]), sin(state[3 * i + 2]), 0};
      for_each_neighbour(s, state, i, visit_local, &c);
      acc += hypot(c.re, c.im) / (double)(c.cnt + 1);
    }
    *R_local = acc / n;
  }
}

/* Philox4x32-10, as published by Salmon et al. (SC'11): multipliers
 * 0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 / 0xBB67AE85. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* ======================================================================
 * VortexArraysSystemPtr (DynamicalSystems/VortexArraysSystemPtr.cpp): the
 * reference's second model.  Distance-dependent alignment mu+ (1 - r^2/xi_a^2)
 * inside xi_a and anti-alignment -4 mu- (r - xi_a)(rho - r)/(rho - xi_a)^2 up
 * to rho (:740-761), and cohesion -kappa sin(atan2(dy, dx) - phi_i) inside xi_r.
 * The cutoffs compare dr = sqrt(dx^2 + dy^2); candidates are the 3x3 stencil
 * of rho-cells (a cohesion partner beyond the stencil is not seen, as in the
 * reference).
 * ====================================================================== */

orc_system *orc_va_create(int n, double L, double velocity, double mu_plus, double mu_minus,
                          double xi_a, double xi_r, double D_phi, double kappa, double rho) {
  orc_system *s = orc_create(n, L, velocity, 0.0, rho, 0.0, D_phi);
  if (!s) return NULL;
  s->va = 1;
  s->mu_plus = mu_plus;
  s->mu_minus = mu_minus;
  s->xi_a = xi_a;
  s->xi_r = xi_r;
  s->kappa = kappa;
  s->anti = (double *)calloc((size_t)n, sizeof(double));
  s->coh = (double *)calloc((size_t)n, sizeof(double));
  s->card1 = (double *)calloc((size_t)n, sizeof(double));
  s->card2 = (double *)calloc((size_t)n, sizeof(double));
  if (!s->anti || !s->coh || !s->card1 || !s->card2) {
    orc_destroy(s);
    return NULL;
  }
  return s;
}

/* AlignmentStrength (VortexArraysSystemPtr.cpp:737-749) */
static double va_strength(const orc_system *s, double r) {
  if (r < s->xi_a) return s->mu_plus * (1.0 - r * r / (s->xi_a * s->xi_a));
  if (r < s->rho)
    return -s->mu_minus * 4.0 * (r - s->xi_a) * (s->rho - r) / (s->rho - s->xi_a) / (s->rho - s->xi_a);
  return 0.0;
}

/* AlignmentStrengthDerivative (VortexArraysSystemPtr.cpp:751-763) */
static double va_strength_derivative(const orc_system *s, double r) {
  if (r < s->xi_a) return s->mu_plus * (-2.0 * r / s->xi_a / s->xi_a);
  if (r < s->rho)
    return -s->mu_minus * 4.0 * (-2.0 * r + s->rho + s->xi_a) / (s->rho - s->xi_a) / (s->rho - s->xi_a);
  return 0.0;
}

/* Every candidate j != i of i with its minimum-image (dx, dy): the 3x3
 * stencil with copy-wrapped positions (VortexArraysSystemPtr.cpp:446-473), or
 * all pairs on the unwrapped stage positions (:164-183). */
typedef void (*va_visit_fn)(void *ctx, int i, int j, double dx, double dy, const double *pos);

static void va_for_each_candidate(orc_system *s, const double *pos, int i, va_visit_fn fn,
                                  void *ctx) {
  if (!orc_uses_cell_list(s)) {
    const double xi = pos[3 * i], yi = pos[3 * i + 1];
    for (int j = 0; j < s->n; ++j) {
      if (j == i) continue;
      double dx, dy;
      orc_min_image(s, xi, yi, pos[3 * j], pos[3 * j + 1], &dx, &dy);
      fn(ctx, i, j, dx, dy, pos);
    }
    return;
  }
  const int nc = s->nc;
  double xi = pos[3 * i], yi = pos[3 * i + 1];
  wrap_if_outside(s, &xi, &yi);
  int cx = cell_coord(s, xi, 0);
  int cy = cell_coord(s, yi, 0);
  for (int q = 0; q < 9; ++q) {
    int jx = adjust_cell(cx + kStencil[q][0], nc);
    int jy = adjust_cell(cy + kStencil[q][1], nc);
    int c = jy * nc + jx;
    for (int p = s->cell_start[c]; p < s->cell_start[c + 1]; ++p) {
      int j = s->cell_items[p];
      if (j == i) continue;
      double xj = pos[3 * j], yj = pos[3 * j + 1];
      wrap_if_outside(s, &xj, &yj);
      double dx, dy;
      orc_min_image(s, xi, yi, xj, yj, &dx, &dy);
      fn(ctx, i, j, dx, dy, pos);
    }
  }
}

/* pass 1 (VortexArraysSystemPtr.cpp:472-488, all pairs :183-199) */
static void va_visit_pass1(void *ctx, int i, int j, double dx, double dy, const double *pos) {
  orc_system *s = (orc_system *)ctx;
  const double phi_i = pos[3 * i + 2], phi_j = pos[3 * j + 2];
  const double dr = sqrt(dx * dx + dy * dy);
  if (dr <= s->xi_a) {
    s->af[i] += va_strength(s, dr) * sin(phi_j - phi_i);
    s->card[i] += 1.0;
  } else if (dr <= s->rho) {
    s->anti[i] += va_strength(s, dr) * sin(phi_j - phi_i);
    s->card1[i] += 1.0;
  }
  if (dr <= s->xi_r) {
    s->coh[i] += -s->kappa * sin(atan2(dy, dx) - phi_i);
    s->card2[i] += 1.0;
  }
}

static void va_reset(orc_system *s) {
  const size_t n = (size_t)s->n;
  memset(s->af, 0, n * sizeof(double));
  memset(s->anti, 0, n * sizeof(double));
  memset(s->coh, 0, n * sizeof(double));
  memset(s->card, 0, n * sizeof(double));
  memset(s->card1, 0, n * sizeof(double));
  memset(s->card2, 0, n * sizeof(double));
}

/* the phase rate of k_next / derivative (VortexArraysSystemPtr.cpp:493-504):
 * written only when the particle has (anti-)alignment partners, then the
 * cohesion mean added on top when it has cohesion partners */
static void va_rate(const orc_system *s, int i, double *out) {
  if ((s->card[i] + s->card1[i]) > 0)
    *out = (s->af[i] + s->anti[i]) / (s->card[i] + s->card1[i]);
  if (s->card2[i] > 0) *out += s->coh[i] / s->card2[i];
}

void orc_va_rhs_rk(orc_system *s, const double *state, const double *k_prev, double *k_next,
                   double k_coef, double dt, int *counts3) {
  const int n = s->n;
  va_reset(s);
  for (int i = 0; i < 3 * n; ++i) s->rk[i] = state[i] + k_coef * dt * k_prev[i];
  if (orc_uses_cell_list(s)) build_linked_list(s, s->rk);
  for (int i = 0; i < n; ++i) {
    va_for_each_candidate(s, s->rk, i, va_visit_pass1, s);
    const double phi_i = s->rk[3 * i + 2];
    k_next[3 * i] = s->v0 * cos(phi_i);
    k_next[3 * i + 1] = s->v0 * sin(phi_i);
    va_rate(s, i, &k_next[3 * i + 2]);
    if (counts3) {
      counts3[3 * i] = (int)s->card[i];
      counts3[3 * i + 1] = (int)s->card1[i];
      counts3[3 * i + 2] = (int)s->card2[i];
    }
  }
}

typedef struct {
  orc_system *s;
  const double *d;
  double *a;
} va_pass2_ctx;

/* pass 2 (VortexArraysSystemPtr.cpp:659-732, all pairs :302-352) */
static void va_visit_pass2(void *vctx, int i, int j, double dx, double dy, const double *pos) {
  va_pass2_ctx *c = (va_pass2_ctx *)vctx;
  orc_system *s = c->s;
  const double *d = c->d;
  const int ii = 3 * i, jj = 3 * j;
  const double phi_i = pos[ii + 2], phi_j = pos[jj + 2];
  const double dr = sqrt(dx * dx + dy * dy);
  const double norm_1 = s->card[i] + s->card1[i];
  const double norm_2 = s->card2[i];
  if ((dr <= s->rho) && (norm_1 > 0.0)) {
    const double cp = cos(phi_j - phi_i);
    const double sp = sin(phi_j - phi_i);
    const double as = va_strength(s, dr);
    const double asd = va_strength_derivative(s, dr);
    c->a[2 * i] += -as * cp / norm_1;
    c->a[2 * i + 1] += ((d[jj] - d[ii]) * asd * dx / dr + (d[jj + 1] - d[ii + 1]) * asd * dy / dr) * sp / norm_1
                       + (d[jj + 2] - d[ii + 2]) * as * cp / norm_1
                       - 2.0 * s->D_phi * sp * as / norm_1;
  }
  if ((dr <= s->xi_r) && (norm_2 > 0.0)) {
    const double cq = cos(atan2(dy, dx) - phi_i);
    const double sq = sin(atan2(dy, dx) - phi_i);
    c->a[2 * i] += s->kappa * cq / norm_2;
    c->a[2 * i + 1] += -s->kappa * ((d[jj] - d[ii]) * (-dy) / dr / dr + (d[jj + 1] - d[ii + 1]) * dx / dr / dr
                                    - d[ii + 2]) * cq / norm_2
                       + s->kappa * s->D_phi * sq / norm_2;
  }
}

void orc_va_rhs_srk(orc_system *s, const double *state, double *derivative, double *additional,
                    int *counts3) {
  const int n = s->n;
  va_reset(s);
  if (orc_uses_cell_list(s)) build_linked_list(s, state);
  for (int i = 0; i < n; ++i) {
    va_for_each_candidate(s, state, i, va_visit_pass1, s);
    const double phi_i = state[3 * i + 2];
    derivative[3 * i] = s->v0 * cos(phi_i);
    derivative[3 * i + 1] = s->v0 * sin(phi_i);
    va_rate(s, i, &derivative[3 * i + 2]);
    if (counts3) {
      counts3[3 * i] = (int)s->card[i];
      counts3[3 * i + 1] = (int)s->card1[i];
      counts3[3 * i + 2] = (int)s->card2[i];
    }
  }
  va_pass2_ctx c = {s, derivative, additional};
  for (int i = 0; i < n; ++i) {
    va_for_each_candidate(s, state, i, va_visit_pass2, &c);
    additional[2 * i] *= sqrt(2.0 * s->D_phi);
  }
}

/* StochasticEulerStepperPtr / StochasticRungeKuttaStepperPtr /
 * RungeKutta4StepperPtr DoStep for VortexArraysSystemPtr
 * (StochasticEulerStepperPtr.hpp:56-76, StochasticRungeKuttaStepperPtr.hpp:70-96,
 * RungeKutta4StepperPtr.cpp:45-63). */
static void va_step(orc_system *s, int stepper, double *state, double dt, const double *noise) {
  const int n = s->n;
  if (stepper == ORC_RK4) {
    double *k1 = s->k[0], *k2 = s->k[1], *k3 = s->k[2], *k4 = s->k[3];
    orc_va_rhs_rk(s, state, k1, k1, 0.0, dt, NULL);
    orc_va_rhs_rk(s, state, k1, k2, 0.5, dt, NULL);
    orc_va_rhs_rk(s, state, k2, k3, 0.5, dt, NULL);
    orc_va_rhs_rk(s, state, k3, k4, 1.0, dt, NULL);
    for (int i = 0; i < n; ++i) {
      int ii = 3 * i;
      state[ii] += (k1[ii] + 2.0 * k2[ii] + 2.0 * k3[ii] + k4[ii]) * dt / 6.0;
      state[ii + 1] += (k1[ii + 1] + 2.0 * k2[ii + 1] + 2.0 * k3[ii + 1] + k4[ii + 1]) * dt / 6.0;
      state[ii + 2] += (k1[ii + 2] + 2.0 * k2[ii + 2] + 2.0 * k3[ii + 2] + k4[ii + 2]) / 6.0 * dt;
    }
    return;
  }
  memset(s->deriv, 0, (size_t)3 * n * sizeof(double));
  memset(s->addl, 0, (size_t)2 * n * sizeof(double));
  orc_va_rhs_srk(s, state, s->deriv, s->addl, NULL);
  const double D = s->D_phi;
  for (int i = 0; i < n; ++i) {
    const double *d = s->deriv + 3 * i;
    const double *a = s->addl + 2 * i;
    if (stepper == ORC_EULER_PTR) {
      double delta_W = sqrt(dt) * noise[i];
      state[3 * i] += d[0] * dt;
      state[3 * i + 1] += d[1] * dt;
      state[3 * i + 2] += d[2] * dt + sqrt(2.0 * D) * delta_W;
    } else {
      double U_1 = noise[2 * i], U_2 = noise[2 * i + 1];
      double delta_W = U_1 * sqrt(dt);
      double delta_Z = 0.5 * dt * sqrt(dt) * (U_1 + U_2 / sqrt(3.0));
      state[3 * i] += d[0] * dt - sqrt(2.0 * D) * d[1] * delta_Z - 0.5 * (d[2] * d[1] + D * d[0]) * dt * dt;
      state[3 * i + 1] += d[1] * dt + sqrt(2.0 * D) * d[0] * delta_Z + 0.5 * (d[2] * d[0] - D * d[1]) * dt * dt;
      state[3 * i + 2] += d[2] * dt + sqrt(2.0 * D) * delta_W + a[0] * delta_Z + 0.5 * a[1] * dt * dt;
    }
  }
}

double orc_va_run(orc_system *s, int stepper, double *state, double t0, double dt, int nsteps,
                  const double *noise) {
  double t = t0;
  const int n = s->n;
  const int per = stepper == ORC_SRK ? 2 * n : (stepper == ORC_EULER_PTR ? n : 0);
  for (int k = 0; k < nsteps; ++k) {
    t += dt;
    va_step(s, stepper, state, dt, noise ? noise + (size_t)k * per : NULL);
    orc_wrap_state(s, state); /* SimulationEnginePtr.cpp:111 */
  }
  return t;
}
