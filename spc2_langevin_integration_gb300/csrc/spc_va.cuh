// VortexArraysSystemPtr neighbour passes (plain FP64), the reference's second
// model (DynamicalSystems/VortexArraysSystemPtr.cpp).
//
// Per candidate pair the model needs the exact distance dr = sqrt(dx^2 + dy^2)
// and, for cohesion, the bearing atan2(dy, dx): pass 1 sums the alignment
// (dr <= xi_a), anti-alignment (xi_a < dr <= rho) and cohesion (dr <= xi_r)
// terms with their three counts (:472-488); pass 2 (the stochastic
// Runge-Kutta form) sums the additional derivative (:695-728) from the pass-1
// derivatives of both particles.  One CTA takes one cell: the candidates of
// its 3x3 stencil (the reference's visiting order, ChimeraSystem-style
// linked list :446-473; all of the system's particles in index order when
// rho > L/4, :164-183) are staged in shared memory, and each thread walks
// them for one particle in order, so every sum keeps the reference's order.
// A float test on cell-relative coordinates drops candidates beyond
// max(rho, xi_r) for certain; every other candidate is decided and evaluated
// in FP64 exactly as the reference writes it.
#pragma once

#include "spc_tile.cuh"

namespace spc {

constexpr int kVAThreads = 64;
constexpr int kVACap = 512;  // candidates staged per round

// AlignmentStrength (VortexArraysSystemPtr.cpp:737-749); the divisions by
// the constants xi_a^2 and w = rho - xi_a use their precomputed reciprocals
// (ddiv_by: the same correctly rounded quotients)
__device__ __forceinline__ double va_strength(const SysConst &sc, double r) {
  if (r < sc.xi_a) return dmul(sc.mu_plus, dsub(1.0, ddiv_by(dmul(r, r), sc.va_xa2, sc.va_rxa2)));
  if (r < sc.rho) {
    const double w = sc.va_w, rw = sc.va_rw;
    return ddiv_by(ddiv_by(dmul(dmul(dmul(-sc.mu_minus, 4.0), dsub(r, sc.xi_a)), dsub(sc.rho, r)), w, rw), w, rw);
  }
  return 0.0;
}

// AlignmentStrengthDerivative (VortexArraysSystemPtr.cpp:751-763)
__device__ __forceinline__ double va_strength_derivative(const SysConst &sc, double r) {
  if (r < sc.xi_a)
    return dmul(sc.mu_plus, ddiv_by(ddiv_by(dmul(-2.0, r), sc.xi_a, sc.va_rxa), sc.xi_a, sc.va_rxa));
  if (r < sc.rho) {
    const double w = sc.va_w, rw = sc.va_rw;
    return ddiv_by(ddiv_by(dmul(dmul(-sc.mu_minus, 4.0), dadd(dadd(dmul(-2.0, r), sc.rho), sc.xi_a)), w, rw),
                   w, rw);
  }
  return 0.0;
}

// Per-particle results of a pass.
struct VAAcc {
  double align, anti, coh;  // pass 1
  int c0, c1, c2;
  double a0, a1;            // pass 2
};

// Fused epilogue of the vortex-arrays passes for the particle at cell-order
// slot p, pool slot q.
template <int KIND>
__device__ void va_epilogue(const KArgs &a, int epi, const SysDesc &sd, int p, int q, double phi,
                            const VAAcc &r) {
  const SysConst &sc = sd.sc;
  const bool live = a.step_off < sd.budget;
  const int i = q - sd.pool_p0;
  const unsigned long long step = sd.step + (unsigned long long)a.step_off;
  const double dt = a.dt;
  double z0 = 0.0, z1 = 0.0;
  const bool draws = (epi == kEpiEulerPtr || epi == kEpiSrk2) && !a.noise && live;
  if (draws) philox_normal2(sd.seed, sd.system_id, step, (uint32_t)i, z0, z1);
  if constexpr (KIND == kKindSin) {
    // k_next / derivative (VortexArraysSystemPtr.cpp:491-504): velocity
    // components always; the phase rate only when there are (anti-)alignment
    // partners, then the cohesion mean added on top
    const double d0 = dmul(sc.v0, cos(phi)), d1 = dmul(sc.v0, sin(phi));
    const int c01 = r.c0 + r.c1;
    auto rate_from = [&](double prev) {
      double v = prev;
      if (c01 > 0) v = ddiv(dadd(r.align, r.anti), (double)c01);
      if (r.c2 > 0) v = dadd(v, ddiv(r.coh, (double)r.c2));
      return v;
    };
    if (epi == kEpiSrk1) {
      a.dphi_s[p] = rate_from(0.0);  // the stepper zero-fills derivative
      a.cnt_s[p] = c01;
      a.va_cnt2[p] = r.c2;
      a.va_vx[p] = d0;
      a.va_vy[p] = d1;
    } else if (epi == kEpiEulerPtr) {
      if (!live) return;
      // StochasticEulerStepperPtr.hpp:56-76
      const double rate = rate_from(0.0);
      const double dW = dmul(a.sdt, noise_at(a, q, 0, z0, z1));
      const double xs = dadd(a.x[q], dmul(d0, dt));
      const double ys = dadd(a.y[q], dmul(d1, dt));
      a.phi[q] = dadd(a.phi[q], dadd(dmul(rate, dt), dmul(sc.s2D, dW)));
      a.x[q] = wrap_1d(xs, sc.rL, sc.L);
      a.y[q] = wrap_1d(ys, sc.rL, sc.L);
    } else if (epi == kEpiRkK || epi == kEpiRk4Combine) {
      if (!live) return;
      const int k = a.kq_out;
      a.kx[k][q] = d0;
      a.ky[k][q] = d1;
      a.kphi[k][q] = rate_from(a.kphi[k][q]);  // the persistent k keeps a stale rate (H5)
      if (epi == kEpiRk4Combine) {
        // RungeKutta4StepperPtr.cpp:57-61
        const double sx_ = dadd(dadd(dadd(a.kx[0][q], dmul(2.0, a.kx[1][q])), dmul(2.0, a.kx[2][q])), a.kx[3][q]);
        const double sy_ = dadd(dadd(dadd(a.ky[0][q], dmul(2.0, a.ky[1][q])), dmul(2.0, a.ky[2][q])), a.ky[3][q]);
        const double sp_ =
            dadd(dadd(dadd(a.kphi[0][q], dmul(2.0, a.kphi[1][q])), dmul(2.0, a.kphi[2][q])), a.kphi[3][q]);
        const double xs = dadd(a.x[q], ddiv(dmul(sx_, dt), 6.0));
        const double ys = dadd(a.y[q], ddiv(dmul(sy_, dt), 6.0));
        a.phi[q] = dadd(a.phi[q], dmul(ddiv(sp_, 6.0), dt));
        a.x[q] = wrap_1d(xs, sc.rL, sc.L);
        a.y[q] = wrap_1d(ys, sc.rL, sc.L);
      }
    }
  } else {
    // additional_derivative[i][0] *= sqrt(2 D) (VortexArraysSystemPtr.cpp:732)
    const double A0 = dmul(r.a0, sc.s2D);
    const double A1 = r.a1;
    const double d0 = a.va_vx[p], d1 = a.va_vy[p], d2 = a.dphi_s[p];
    if (epi == kEpiSrk2Out) {
      a.out_d[3 * (size_t)q] = d0;
      a.out_d[3 * (size_t)q + 1] = d1;
      a.out_d[3 * (size_t)q + 2] = d2;
      a.out_a[2 * (size_t)q] = A0;
      a.out_a[2 * (size_t)q + 1] = A1;
    } else {
      if (!live) return;
      // StochasticRungeKuttaStepperPtr.hpp:70-96 (no natural frequencies)
      const double U1 = noise_at(a, q, 0, z0, z1), U2 = noise_at(a, q, 1, z0, z1);
      const double sdt = a.sdt;
      const double dW = dmul(U1, sdt);
      const double dZ = dmul(dmul(dmul(0.5, dt), sdt), dadd(U1, ddiv_by(U2, kSqrt3, kRcpSqrt3)));
      const double D = sc.D;
      const double s2D = sc.s2D;
      const double dtdt_x = dmul(dmul(dmul(0.5, dadd(dmul(d2, d1), dmul(D, d0))), dt), dt);
      const double xs = dadd(a.x[q], dsub(dsub(dmul(d0, dt), dmul(dmul(s2D, d1), dZ)), dtdt_x));
      const double dtdt_y = dmul(dmul(dmul(0.5, dsub(dmul(d2, d0), dmul(D, d1))), dt), dt);
      const double ys = dadd(a.y[q], dadd(dadd(dmul(d1, dt), dmul(dmul(s2D, d0), dZ)), dtdt_y));
      const double ps = dadd(a.phi[q], dadd(dadd(dadd(dmul(d2, dt), dmul(s2D, dW)), dmul(A0, dZ)),
                                            dmul(dmul(dmul(0.5, A1), dt), dt)));
      a.x[q] = wrap_1d(xs, sc.rL, sc.L);
      a.y[q] = wrap_1d(ys, sc.rL, sc.L);
      a.phi[q] = ps;
    }
  }
}

template <int KIND>
struct VAStage {
  float2 xy[kVACap];  // x+shift, y+shift (prefilter; cell-list systems)
  double phi[kVACap];
  int slot[kVACap];
  // pass 2: the candidates' pass-1 derivatives
  double vx[KIND == kKindCos2 ? kVACap : 1], vy[KIND == kKindCos2 ? kVACap : 1];
  double dd[KIND == kKindCos2 ? kVACap : 1];
};

template <int KIND>
__global__ void __launch_bounds__(kVAThreads) k_va_pass(KArgs a, int epi) {
  __shared__ VAStage<KIND> sm;
  const int tid = threadIdx.x;
  const int n_all = a.n_active;
  for (int c = a.va_c0 + blockIdx.x; c < a.va_c1; c += gridDim.x) {
    const int cb = a.cell_start[c], ce = a.cell_start[c + 1];
    if (cb == ce) continue;
    const SysDesc &sd = a.sys[a.sys_of_c[c]];
    const SysConst &sc = sd.sc;
    const bool ap = sc.allpairs != 0;
    Stencil st;
    if (ap) {  // one cell holding the whole system, in index order
#pragma unroll
      for (int k = 0; k < 9; ++k) st.start[k] = cb;
      st.prefix[0] = 0;
#pragma unroll
      for (int k = 1; k < 10; ++k) st.prefix[k] = ce - cb;
    } else {
      stencil_of(a, sd, c, st);
    }
    const int total = st.prefix[9];
    const int rounds = (total + kVACap - 1) / kVACap;
    for (int ig = cb; ig < ce; ig += kVAThreads) {
      const int p = ig + tid;
      const bool valid = p < ce;
      double xi = 0.0, yi = 0.0, phii = 0.0;
      float fx = 0.0f, fy = 0.0f;
      double vxi = 0.0, vyi = 0.0, ddi = 0.0, norm1 = 0.0, norm2 = 0.0, rn1 = 1.0, rn2 = 1.0;
      if (valid) {
        xi = a.sx[p];
        yi = a.sy[p];
        phii = a.sphi[p];
        if (!ap) {
          const float2 f = a.fxy[p];
          fx = f.x;
          fy = f.y;
        }
        if constexpr (KIND == kKindCos2) {
          vxi = a.va_vx[p];
          vyi = a.va_vy[p];
          ddi = a.dphi_s[p];
          norm1 = (double)a.cnt_s[p];   // neighborhood_cardinality_[i][0] + [i][1]
          norm2 = (double)a.va_cnt2[p]; // neighborhood_cardinality_[i][2]
          rn1 = drcp(norm1);            // used only when norm1 > 0 (ddiv_by)
          rn2 = drcp(norm2);
        }
      }
      const int self = (ap ? 0 : st.prefix[4]) + (p - cb);
      VAAcc r{0.0, 0.0, 0.0, 0, 0, 0, 0.0, 0.0};
      int kr = 0;  // pairs within rho so far: the index of this particle's pair records
      for (int rr = 0; rr < rounds; ++rr) {
        const int rlo = rr * kVACap, rcnt = min(kVACap, total - rlo);
        if (rounds > 1 || ig == cb) {
          __syncthreads();
          for (int k = tid; k < rcnt; k += blockDim.x) {
            int q;
            const int pj = slot_of(st, rlo + k, q);
            if (!ap) {
              const float2 f = a.fxy[pj];
              sm.xy[k] = make_float2(f.x + shift_x(q, sc.cell_f), f.y + shift_y(q, sc.cell_f));
            }
            sm.phi[k] = a.sphi[pj];
            sm.slot[k] = pj;
            if constexpr (KIND == kKindCos2) {
              sm.vx[k] = a.va_vx[pj];
              sm.vy[k] = a.va_vy[pj];
              sm.dd[k] = a.dphi_s[pj];
            }
          }
          __syncthreads();
        }
        if (!valid) continue;
        for (int j = 0; j < rcnt; ++j) {
          if (rlo + j == self) continue;
          if (!ap) {
            const float2 cj = sm.xy[j];
            const float ex = cj.x - fx, ey = cj.y - fy;
            if (fmaf(ex, ex, ey * ey) > sc.va_r2) continue;  // beyond rho and xi_r for certain
          }
          // ClassAEffectiveParticleDistance on the (copy-wrapped) stage positions
          const int pj = sm.slot[j];
          const double dx = min_image_1d(dsub(a.sx[pj], xi), sc.rL, sc.L);
          const double dy = min_image_1d(dsub(a.sy[pj], yi), sc.rL, sc.L);
          const double dr = dsqrt(dadd(dmul(dx, dx), dmul(dy, dy)));
          const double phij = sm.phi[j];
          // a pair within rho has a record for the second SRK pass (single
          // systems): the same strength, derivative, sin and cos bit for bit
          const bool rho_pair = dr <= sc.rho;
          double *rec = (rho_pair && a.vacache && kr < a.vacap) ? a.vacache + ((size_t)kr * n_all + p) * 4 : nullptr;
          kr += rho_pair ? 1 : 0;
          if constexpr (KIND == kKindSin) {
            // VortexArraysSystemPtr.cpp:475-488
            if (dr <= sc.xi_a || rho_pair) {
              double as, sn;
              if (rec) {
                double cn;
                sincos(dsub(phij, phii), &sn, &cn);  // the bits of sin and cos
                as = va_strength(sc, dr);
                rec[0] = as;
                rec[1] = va_strength_derivative(sc, dr);
                rec[2] = sn;
                rec[3] = cn;
              } else {
                as = va_strength(sc, dr);
                sn = sin(dsub(phij, phii));
              }
              if (dr <= sc.xi_a) {
                r.align = dadd(r.align, dmul(as, sn));
                ++r.c0;
              } else {
                r.anti = dadd(r.anti, dmul(as, sn));
                ++r.c1;
              }
            }
            if (dr <= sc.xi_r) {
              r.coh = dadd(r.coh, dmul(-sc.kappa, sin(dsub(atan2(dy, dx), phii))));
              ++r.c2;
            }
          } else {
            // VortexArraysSystemPtr.cpp:706-728
            if (rho_pair && (norm1 > 0.0)) {
              double cp, sp, as, asd;
              if (rec) {  // the first pass's values
                as = rec[0];
                asd = rec[1];
                sp = rec[2];
                cp = rec[3];
              } else {
                cp = cos(dsub(phij, phii));
                sp = sin(dsub(phij, phii));
                as = va_strength(sc, dr);
                asd = va_strength_derivative(sc, dr);
              }
              // every quotient by norm1 or dr as ddiv would give it (ddiv_by)
              const double rdr = drcp(dr);
              r.a0 = dadd(r.a0, ddiv_by(dmul(-as, cp), norm1, rn1));
              const double gx = ddiv_by(dmul(dmul(dsub(sm.vx[j], vxi), asd), dx), dr, rdr);
              const double gy = ddiv_by(dmul(dmul(dsub(sm.vy[j], vyi), asd), dy), dr, rdr);
              const double t1 = ddiv_by(dmul(dadd(gx, gy), sp), norm1, rn1);
              const double t2 = ddiv_by(dmul(dmul(dsub(sm.dd[j], ddi), as), cp), norm1, rn1);
              const double t3 = ddiv_by(dmul(dmul(dmul(2.0, sc.D), sp), as), norm1, rn1);
              r.a1 = dadd(r.a1, dsub(dadd(t1, t2), t3));
            }
            if ((dr <= sc.xi_r) && (norm2 > 0.0)) {
              const double th = atan2(dy, dx);
              const double cq = cos(dsub(th, phii)), sq = sin(dsub(th, phii));
              const double rdr = drcp(dr);
              r.a0 = dadd(r.a0, ddiv_by(dmul(sc.kappa, cq), norm2, rn2));
              const double inner =
                  dsub(dadd(ddiv_by(ddiv_by(dmul(dsub(sm.vx[j], vxi), -dy), dr, rdr), dr, rdr),
                            ddiv_by(ddiv_by(dmul(dsub(sm.vy[j], vyi), dx), dr, rdr), dr, rdr)),
                       ddi);
              const double u1 = ddiv_by(dmul(dmul(-sc.kappa, inner), cq), norm2, rn2);
              const double u2 = ddiv_by(dmul(dmul(sc.kappa, sc.D), sq), norm2, rn2);
              r.a1 = dadd(r.a1, dadd(u1, u2));
            }
          }
        }
      }
      if (valid) va_epilogue<KIND>(a, epi, sd, p, a.pidx[p], phii, r);
    }
  }
}

}  // namespace spc
