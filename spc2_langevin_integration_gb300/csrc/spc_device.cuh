// Device helpers shared by every kernel of the particle-update path.
//
// Parity-critical double arithmetic is written with the _rn intrinsics so
// that nvcc never fuses a product into an add: the reference's C++ is plain
// unfused IEEE double, and cutoff decisions must come out bit-identical.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "spc_fixed.h"

namespace spc {

constexpr int kWarp = 32;

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// a / b rounded to nearest, for a divisor b used many times, from its
// reciprocal y = RN(1 / b) computed once: q = RN(a y) is within an ulp of
// a / b, the remainder a - q b is exact in one fused multiply-add, and
// RN(q + (a - q b) y) = RN(a / b) (the final correction step of
// Newton-Raphson division, P. Markstein, "Computation of elementary functions
// on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990).
// Bitwise equal to ddiv(a, b) for the finite nonzero divisors of these
// kernels (spc_check_division checks it on the device); it replaces two
// correctly rounded divisions per pair by a multiply and two fused
// multiply-adds on the FP64 pipe.
__device__ __forceinline__ double ddiv_by(double a, double b, double y) {
  const double q = __dmul_rn(a, y);
  const double r = __fma_rn(-q, b, a);
  return __fma_rn(r, y, q);
}
__device__ __forceinline__ double drcp(double b) { return __drcp_rn(b); }
// sqrt(3) and RN(1 / sqrt(3)) for the SRK update's U2 / sqrt(3) (by ddiv_by,
// bitwise the division)
constexpr double kSqrt3 = 1.7320508075688772;
constexpr double kRcpSqrt3 = 1.0 / kSqrt3;
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }

// FP32X fixed point.  A value v with |v| <= 1 is held as the integer
// RN(v 2^52); a staging round of at most 1024 candidates sums to less than
// 2^62 in magnitude, so the integer sums are exact, and the conversion back
// (one rounding to double) is the only error of a round's sum.
constexpr int kXQ = 52;
// v 2^q is exact (a power-of-two scaling of a normal result), then rounded
// to the nearest integer
__device__ __forceinline__ long long to_fixed(double v, int q) {
  return __double2ll_rn(__dmul_rn(v, pow2i(q)));
}
__device__ __forceinline__ double from_fixed(long long v, int q) { return fixed_to_double(v, q); }
// A particle's whole sum over several staging rounds is kept in 128 bits, so
// it is one exact integer whatever the kernel's round size, and converted to
// double once: one rounding when it fits 64 bits (always below 2^11
// neighbours), else a fixed two-step conversion.  Either way the result
// depends on the integer alone.
__device__ __forceinline__ double from_fixed128(__int128 v, int q) {
  const long long lo64 = (long long)v;
  if ((__int128)lo64 == v) return fixed_to_double(lo64, q);
  const long long hi = (long long)(v >> 64);
  const unsigned long long lo = (unsigned long long)v;
  return __dmul_rn(__fma_rn(__ll2double_rn(hi), 18446744073709551616.0, __ull2double_rn(lo)), pow2i(-q));
}
// c += v.x, s += v.y when p: predicated 64-bit adds, so a candidate loop whose
// lanes disagree on p runs straight through instead of branching around the
// adds of each candidate
__device__ __forceinline__ void add2_if(long long &c, long long &s, longlong2 v, bool p) {
  asm("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %4, 0;\n\t@q add.s64 %0, %0, %2;\n\t@q add.s64 %1, %1, %3;\n\t}"
      : "+l"(c), "+l"(s)
      : "l"(v.x), "l"(v.y), "r"((int)p));
}
// the same for float sums: c += x, s += y when p (each rounded to nearest,
// as the plain adds)
__device__ __forceinline__ void addf2_if(float &c, float &s, float x, float y, bool p) {
  asm("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %4, 0;\n\t@q add.rn.f32 %0, %0, %2;\n\t@q add.rn.f32 %1, %1, %3;\n\t}"
      : "+f"(c), "+f"(s)
      : "f"(x), "f"(y), "r"((int)p));
}
// c = fma(d, x, c), s = fma(d, y, s) when p
__device__ __forceinline__ void fmaf2_if(float &c, float &s, float d, float x, float y, bool p) {
  asm("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %5, 0;\n\t@q fma.rn.f32 %0, %2, %3, %0;\n\t@q fma.rn.f32 %1, %2, %4, %1;\n\t}"
      : "+f"(c), "+f"(s)
      : "f"(d), "f"(x), "f"(y), "r"((int)p));
}

// Per-system constants, the reference's ChimeraSystem / PeriodicBoundaryConditions
// members (ChimeraSystem.cpp:19-33, PeriodicBoundaryConditions.cpp:13-14).
struct SysConst {
  int n;          // particles
  int nc;         // num_subcells_ = int(kL / rho)
  int ncell;      // nc * nc
  int allpairs;   // rho > 0.25 L: EvaluateInteractionsWithAllPairs (ChimeraSystem.cpp:90-98)
  double L, rL;   // x_size_, x_rsize_ = 1.0 / x_size
  double rho;     // rho_
  double rho2;    // rho_squared_ = rho * rho
  double v0, sigma, alpha, D;
  double cell;    // cell side L / nc, origin of the float prefilter coordinates
  float cell_f;
  float lo2, hi2; // prefilter: float dr^2 < lo2 => inside, > hi2 => outside, else decide in FP64
  int exact_all;  // decide every candidate in FP64
  int L_pow2;     // L is a power of two: x / L == x * (1 / L) exactly
  float cos_a, sin_a;  // FP32C: cos(alpha), sin(alpha) rounded to float
  // FP32X: cos(alpha), sin(alpha) in double, and the fixed-point exponent of
  // the phase-rate-weighted sums of the SRK second pass (sum_j d_j cos phi_j,
  // sum_j d_j sin phi_j): 2^xq2 per unit, |d_j| <= |sigma| < 2^(52 - xq2)
  double cos_ad, sin_ad;
  int xq2;
  double s2D;     // sqrt(2 D), rounded once (the update's per-particle factor)
  // Verlet rows (vR = 0: the system uses the cell-list passes)
  int vR;         // stencil radius in cells, ceil(r_max / cell)
  float vr2;      // build: candidates with float dr^2 <= vr2 (r_max^2 plus a margin) are listed
  double vdisp2;  // a displacement with dr^2 > vdisp2 (about (skin / 2)^2) forces a rebuild
  // VortexArraysSystemPtr (va = 1): v0 is velocity_, D the rotational diffusion
  int va;
  double mu_plus, mu_minus, xi_a, xi_r, kappa;
  float va_r2;    // float dr^2 above this: beyond rho and xi_r for certain
  // vortex arrays: w = rho - xi_a and xi_a^2 as the model computes them, and
  // the reciprocals of w, xi_a and xi_a^2 rounded to nearest (ddiv_by)
  double va_w, va_xa2, va_rw, va_rxa, va_rxa2;
};

// PeriodicBoundaryConditions::ClassAEffectiveParticleDistance (PeriodicBoundaryConditions.cpp:22-35):
// d -= static_cast<int>(d * 2.0 * rL) * L
__device__ __forceinline__ double min_image_1d(double d, double rL, double L) {
  const int k = __double2int_rz(dmul(dmul(d, 2.0), rL));
  return dsub(d, dmul(__int2double_rn(k), L));
}

// The reference's cutoff test dr^2 <= rho^2 on two (already wrapped) positions
// (ChimeraSystem.cpp:407-410), operation for operation.
__device__ __forceinline__ bool exact_within(const SysConst &sc, double xi, double yi, double xj,
                                             double yj) {
  const double dx = min_image_1d(dsub(xj, xi), sc.rL, sc.L);
  const double dy = min_image_1d(dsub(yj, yi), sc.rL, sc.L);
  const double dr2 = dadd(dmul(dx, dx), dmul(dy, dy));
  return dr2 <= sc.rho2;
}

// ApplyPeriodicBoundaryConditions (PeriodicBoundaryConditions.cpp:117-121): x - floor(x * rL) * L.
// When 0 <= x * rL < 1 (an unsigned compare of the bits; -0.0 and NaN fail it)
// floor gives +0.0 and x - 0.0 * L is x itself, so the result is returned
// without the floor, the product and the difference.
__device__ __forceinline__ double wrap_1d(double x, double rL, double L) {
  const double t = dmul(x, rL);
  if ((unsigned long long)__double_as_longlong(t) < 0x3FF0000000000000ull) return x;
  return dsub(x, dmul(floor(t), L));
}

// The conditional copy-wrap inside the force loops (ChimeraSystem.cpp:299-302):
// both coordinates are wrapped when either is outside [0, L).
__device__ __forceinline__ void wrap_if_outside(const SysConst &sc, double &x, double &y) {
  if (x < 0.0 || x >= sc.L || y < 0.0 || y >= sc.L) {
    const double xw = wrap_1d(x, sc.rL, sc.L);
    const double yw = wrap_1d(y, sc.rL, sc.L);
    x = xw;
    y = yw;
  }
}

// int(x / x_size_ * num_subcells_x_) (ChimeraSystem.cpp:304-305).  An index
// outside [0, nc) (x within an ulp of L) is clamped; *clamped is set.
__device__ __forceinline__ int cell_coord(const SysConst &sc, double x, int &clamped) {
  // for a power-of-two L the scaling by 1/L is exact, so it equals the division
  const double q = sc.L_pow2 ? dmul(x, sc.rL) : ddiv(x, sc.L);
  int c = __double2int_rz(dmul(q, (double)sc.nc));
  if (c < 0) {
    c = 0;
    clamped = 1;
  } else if (c >= sc.nc) {
    c = sc.nc - 1;
    clamped = 1;
  }
  return c;
}

// AdjustNeighboringCellToPeriodicBoundaries (ChimeraSystem.cpp:905-922)
__device__ __forceinline__ int adjust_cell(int c, int nc) {
  return c < 0 ? nc - 1 : (c >= nc ? 0 : c);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy
// as 1, 2, 3", SC'11): counter-based, so every (particle, step) draw is a pure
// function of (seed, system, step, particle) and needs no stored RNG state.
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Two standard normals for (particle i, step) by Box-Muller on two 53-bit
// uniforms; u1 in (0, 1] so the logarithm is finite.
__device__ __forceinline__ void philox_normal2(uint64_t seed, uint32_t system_id, uint64_t step,
                                               uint32_t i, double &z0, double &z1) {
  const U4 o = philox4x32_10(U4{i, system_id, (uint32_t)step, (uint32_t)(step >> 32)},
                             (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint64_t a = ((((uint64_t)o.x) << 32) | o.y) >> 11;
  const uint64_t b = ((((uint64_t)o.z) << 32) | o.w) >> 11;
  const double u1 = (double)(a + 1) * 0x1.0p-53;
  const double u2 = (double)b * 0x1.0p-53;
  const double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  z0 = r * c;
  z1 = r * s;
}

// Float form of the same draw for the FP32-compensated path: single-precision
// Box-Muller (the double version's log/sqrt/sincospi run on GB300's 1/64-rate
// FP64 pipe) on the same two 53-bit integers, each rounded once to float, so
// that the result keeps float's RELATIVE precision at both ends of u1:
// * u1 < 1/2 (the normal's tail, steep in u1): log of u1 = (a + 1) 2^-53;
// * u1 >= 1/2 (near-zero radii, where log u1 ~ u1 - 1): log1p(-e) of
//   e = 1 - u1 = (2^53 - 1 - a) 2^-53, exact in integers before the rounding.
// (A 24-bit fixed-point u1 differs from the 53-bit one by up to 2^-24
// absolute, which moves a tail draw by ~1e-5 relative: that error dominated
// the FP32C form's drift from FP64.)  The angle is taken as pi*v with
// v = 2*u2 - 1 in [-1, 1), exact in integers before the rounding, and
// sinpi / cospi(v + 1) = -sinpi / -cospi(v).
__device__ __forceinline__ void philox_normal2_f(uint64_t seed, uint32_t system_id, uint64_t step,
                                                 uint32_t i, float &z0, float &z1) {
  const U4 o = philox4x32_10(U4{i, system_id, (uint32_t)step, (uint32_t)(step >> 32)},
                             (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint64_t a = ((((uint64_t)o.x) << 32) | o.y) >> 11;
  const uint64_t b = ((((uint64_t)o.z) << 32) | o.w) >> 11;
  const float lnu = a < (1ull << 52) ? logf((float)(a + 1) * 0x1.0p-53f)
                                     : log1pf(-(float)((1ull << 53) - 1 - a) * 0x1.0p-53f);
  const float v = (float)((long long)b - (1ll << 52)) * 0x1.0p-52f;
  const float r = sqrtf(-2.0f * lnu);
  float s, c;
  sincospif(v, &s, &c);
  z0 = -r * c;
  z1 = -r * s;
}

// Error word bits reported through spc_diagnostics.
enum : unsigned long long {
  kErrNone = 0,
  kErrVerletOverflow = 1ull << 0,  // a Verlet row exceeded its capacity
  kErrNoiseMissing = 1ull << 1,
};

}  // namespace spc
