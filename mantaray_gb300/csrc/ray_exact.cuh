// ray_exact.cuh -- the reference's right-hand side on the GPU.
//
// Two forms of WaveRayPath::odes (src/wave_ray_path.rs:118-150) over the same
// bit-exact field lookups (lookup.cuh):
//  - RhsLibm: the reference's expression, operation for operation, with its
//    calls to sqrt, atan2, cos, sin, cosh, tanh and sinh (CUDA's versions,
//    within an ulp or two of glibc's; cos and sin of the one angle from
//    sincos, and each call the reference repeats on the same argument made
//    once);
//  - RhsIdentity: the same quantities through exact identities that need
//    fewer FP64 instructions -- cos(atan2(ky, kx)) = kx/k,
//    sin(atan2(ky, kx)) = ky/k, and with a = kh, q = exp(-2a) from the single
//    value m = -expm1(-2a) = 1 - q, and w = 1/(m (1 + q)):
//      tanh a = m / (1 + q),  a / cosh^2 a = 4 a q / (1 + q)^2,
//      1 / (sinh a cosh a) = 4 q w,
//    sqrt(g k tanh) and 1/sqrt(g k tanh) from one rsqrt, 1/k from another,
//    and products and sums contracted into FMAs (kFma; the RK4 update too).
//    Each quantity differs from the libm form by a few ulps, except where
//    exp(-2kh) falls below the rounding of 1 - exp(-2kh) (kh > ~18): q then
//    comes out 0 (or a multiple of 2^-53) instead of its true value below
//    1e-16, so the refraction term f ~ q is off by up to that amount -- a
//    change of k below one ulp of kx, ky per step.  Beyond kh = 22 (where
//    expm1 rounds to exactly -1) the deep-water forms are taken directly:
//    c_g = (g/2) / sqrt(g k) and no refraction term, without the expm1, the
//    reciprocal and the products by zero.
// Both read the field values through the exact lookups, convert between f32
// and f64 on the integer pipe (bits.h) and test NaN / zero on bit patterns,
// which gives the same values as the conversion and comparison instructions.
// Compiled with -fmad=false: the reference's arithmetic is never contracted;
// RhsIdentity's FMAs are explicit fma() calls.
#pragma once

#include <math.h>

#include "lookup.cuh"

namespace mr {

constexpr double kG = 9.8;  // src/wave_ray_path.rs:23

struct RhsLibm {
  static constexpr bool kFma = false;
  // WaveRayPath::odes with group_velocity (:177-188) and dkdt_bathy
  // (:207-216) inlined in the reference's order.
  template <typename Cache>
  __device__ __forceinline__ static int odes(const BathyDev &b, const CurrentDev &c, double x,
                                             double y, double kx, double ky, double out[4],
                                             Cache *L) {
    float hg[3];
    int e = depth_and_gradient<Cache>(b, d2f(x), d2f(y), hg, L);
    if (e) return e;
    const double h = f2d(hg[0]);
    const double dhdx = f2d(hg[1]);
    const double dhdy = f2d(hg[2]);
    double cur[6];
    e = current_and_gradient<Cache>(c, x, y, cur, L);
    if (e) return e;
    const double k = sqrt(kx * kx + ky * ky);
    const double theta = atan2(ky, kx);
    // kh, cosh(kh), tanh(kh) and sqrt(g k tanh(kh)) appear in both
    // group_velocity and dkdt_bathy: each is evaluated once (the same
    // function of the same argument gives the same value, and k * kG equals
    // kG * k exactly, so sqrt(k * kG * th) is sqrt(kG * k * tanh(kh)))
    const double kh = k * h;
    const double ch = cosh(kh);
    const double th = tanh(kh);
    const double sq = sqrt(kG * k * th);
    double cg;
    if (h <= 0.0) {
      cg = f64_nan();
    } else {
      if (k <= 0.0) return RHS_ARGUMENT_OUT_OF_BOUNDS;
      cg = (kG / 2.0) * ((th + kh / (ch * ch)) / sq);
    }
    double st, ct;
    sincos(theta, &st, &ct);
    const double cgx = cg * ct + cur[0];
    const double cgy = cg * st + cur[1];
    const double f = (-0.5) * k * 1.0 / sinh(kh) * 1.0 / ch * sq;
    out[0] = cgx;
    out[1] = cgy;
    out[2] = f * dhdx - kx * cur[2] - ky * cur[4];
    out[3] = f * dhdy - kx * cur[3] - ky * cur[5];
    return RHS_OK;
  }
};

struct RhsIdentity {
  static constexpr bool kFma = true;
  template <typename Cache>
  __device__ __forceinline__ static int odes(const BathyDev &b, const CurrentDev &c, double x,
                                             double y, double kx, double ky, double out[4],
                                             Cache *L) {
    float hg[3];
    int e = depth_and_gradient<Cache>(b, d2f(x), d2f(y), hg, L);
    if (e) return e;
    double cur[6];
    e = current_and_gradient<Cache>(c, x, y, cur, L);
    if (e) return e;
    const double h = f2d(hg[0]);
    const double k2 = fma(kx, kx, ky * ky);
    const double rk = rsqrt(k2);                    // 1/k
    const double k = k2 * rk;
    // group_velocity's k <= 0 error (h > 0 or NaN): k is >= 0 or NaN here
    if (!(hg[0] <= 0.0f) && (__double_as_longlong(k) << 1) == 0) return RHS_ARGUMENT_OUT_OF_BOUNDS;
    const double a = k * h;
    const double gk = kG * k;
    // Deep water, 22 < a < 1e300: exp(-2a) < 8e-20, far below half an ulp
    // of 1, so -expm1(-2a) rounds to exactly 1: tanh a = 1 and the terms in
    // exp(-2a) (a / cosh^2 a, the refraction factor f) are exactly 0.  The
    // range is tested on the bit pattern: for doubles of either sign, NaN
    // included, signed 64-bit order of the bits gives the same answer as
    // the two comparisons, on the integer pipe.  The deep-water form also
    // needs finite gradients (a NaN one makes the refraction term NaN, which
    // stops the ray as in the reference).
    const long long ab = __double_as_longlong(a);
    const uint32_t gx = bits_of(hg[1]), gy = bits_of(hg[2]);
    const bool deep = ab > 0x4036000000000000ll /* 22.0 */ &&
                      ab < 0x7e37e43c8800759cll /* 1e300 */ &&
                      (gx & 0x7f800000u) != 0x7f800000u && (gy & 0x7f800000u) != 0x7f800000u;
    // Deep-water lanes skip the expm1, the reciprocal and the products by
    // zero.  When every converged lane is in deep water the warp takes the
    // deep-water form alone; otherwise every operation but those is shared,
    // so a warp whose rays are in both regimes runs the general form once
    // rather than both forms.  With tanh a = 1 the shared operations give
    // the deep-water form's bits (gkt = g k, c_g = (g/2) rs), so a lane's
    // result does not depend on its neighbours.  The refraction term is
    // dropped rather than added as a signed zero.
    if (__all_sync(__activemask(), deep)) {
      const double rs = rsqrt(gk);                  // 1 / sqrt(g k)
      const double cg = (kG / 2.0) * rs;
      out[0] = fma(cg, kx * rk, cur[0]);
      out[1] = fma(cg, ky * rk, cur[1]);
      out[2] = -fma(kx, cur[2], ky * cur[4]);
      out[3] = -fma(kx, cur[3], ky * cur[5]);
      return RHS_OK;
    }
    double gkt = gk, fac = 1.0, fq = 0.0;
    if (!deep) {
      const double m = -expm1(-2.0 * a);            // 1 - q
      const double q = 1.0 - m;                     // exp(-2a)
      const double w = __drcp_rn(m * (2.0 - m));    // 1 / (m (1 + q))
      const double r = m * w;                       // 1 / (1 + q)
      const double th = m * r;                      // tanh a
      const double q4 = 4.0 * q;
      gkt = gk * th;
      fac = fma(a * q4, r * r, th);                 // tanh a + a / cosh^2 a
      fq = q4 * w;                                  // 1 / (sinh a cosh a)
    }
    const double rs = rsqrt(gkt);                   // 1 / sqrt(g k tanh)
    double cgr = rs, f = 0.0;
    if (!deep) {
      cgr = fac * rs;
      f = (-0.5 * k) * (fq * (gkt * rs));
    }
    double cg = (kG / 2.0) * cgr;
    if (hg[0] <= 0.0f) cg = f64_nan();
    out[0] = fma(cg, kx * rk, cur[0]);
    out[1] = fma(cg, ky * rk, cur[1]);
    double t2 = -fma(kx, cur[2], ky * cur[4]);
    double t3 = -fma(kx, cur[3], ky * cur[5]);
    if (!deep) {
      t2 = fma(f, f2d(hg[1]), t2);
      t3 = fma(f, f2d(hg[2]), t3);
    }
    out[2] = t2;
    out[3] = t3;
    return RHS_OK;
  }
};

// impl System::system (src/wave_ray_path.rs:220-234): errors become NaN.
// Cache: NoCache, or LookupCache with the lane's last cells (lookup.cuh).
template <typename Rhs, typename Cache = NoCache>
__device__ __forceinline__ void system(const BathyDev &b, const CurrentDev &c, const double s[4],
                                       double ds[4], Cache *L = nullptr) {
  if (Rhs::odes(b, c, s[0], s[1], s[2], s[3], ds, L) != RHS_OK) {
    ds[0] = ds[1] = ds[2] = ds[3] = f64_nan();
  }
}

__device__ __forceinline__ bool all_nan4(const double v[4]) {
  return nan_bits(v[0]) && nan_bits(v[1]) && nan_bits(v[2]) && nan_bits(v[3]);
}

}  // namespace mr
