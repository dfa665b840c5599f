// ray_exact.cuh -- the reference's right-hand side on the GPU.
//
// Two forms of WaveRayPath::odes (src/wave_ray_path.rs:118-150) over the same
// bit-exact field lookups (lookup.cuh):
//  - RhsLibm: the reference's expression, operation for operation, with its
//    calls to sqrt, atan2, cos, sin, cosh, tanh and sinh (CUDA's versions,
//    within an ulp or two of glibc's);
//  - RhsIdentity: the same quantities through exact identities that need
//    fewer FP64 instructions -- cos(atan2(ky, kx)) = kx/k,
//    sin(atan2(ky, kx)) = ky/k, and tanh, kh/cosh^2 and 1/(sinh cosh) of kh
//    from the single value m = -expm1(-2kh) = 1 - exp(-2kh):
//      tanh = m/(2-m),  kh/cosh^2 = 4 kh (1-m)/(2-m)^2,
//      1/(sinh cosh) = 4 (1-m)/(m (2-m)),
//    and sqrt(g k tanh) and 1/sqrt(g k tanh) from one rsqrt.  Each quantity
//    differs from the libm form by a few ulps.
// Compiled with -fmad=false (no contraction of the reference's arithmetic).
#pragma once

#include <math.h>

#include "lookup.cuh"

namespace mr {

constexpr double kG = 9.8;  // src/wave_ray_path.rs:23

struct RhsLibm {
  // WaveRayPath::odes with group_velocity (:177-188) and dkdt_bathy
  // (:207-216) inlined in the reference's order.
  __device__ __forceinline__ static int odes(const BathyDev &b, const CurrentDev &c, double x,
                                             double y, double kx, double ky, double out[4]) {
    float hg[3];
    int e = depth_and_gradient(b, __double2float_rn(x), __double2float_rn(y), hg);
    if (e) return e;
    const double h = static_cast<double>(hg[0]);
    const double dhdx = static_cast<double>(hg[1]);
    const double dhdy = static_cast<double>(hg[2]);
    double cur[6];
    e = current_and_gradient(c, x, y, cur);
    if (e) return e;
    const double k = sqrt(kx * kx + ky * ky);
    const double theta = atan2(ky, kx);
    double cg;
    if (h <= 0.0) {
      cg = f64_nan();
    } else {
      if (k <= 0.0) return RHS_ARGUMENT_OUT_OF_BOUNDS;
      const double kh = k * h;
      const double ch = cosh(kh);
      const double th = tanh(kh);
      cg = (kG / 2.0) * ((th + kh / (ch * ch)) / sqrt(k * kG * th));
    }
    const double cgx = cg * cos(theta) + cur[0];
    const double cgy = cg * sin(theta) + cur[1];
    const double kh = k * h;
    const double f = (-0.5) * k * 1.0 / sinh(kh) * 1.0 / cosh(kh) * sqrt(kG * k * tanh(kh));
    out[0] = cgx;
    out[1] = cgy;
    out[2] = f * dhdx - kx * cur[2] - ky * cur[4];
    out[3] = f * dhdy - kx * cur[3] - ky * cur[5];
    return RHS_OK;
  }
};

struct RhsIdentity {
  __device__ __forceinline__ static int odes(const BathyDev &b, const CurrentDev &c, double x,
                                             double y, double kx, double ky, double out[4]) {
    float hg[3];
    int e = depth_and_gradient(b, __double2float_rn(x), __double2float_rn(y), hg);
    if (e) return e;
    const double h = static_cast<double>(hg[0]);
    double cur[6];
    e = current_and_gradient(c, x, y, cur);
    if (e) return e;
    const double k2 = kx * kx + ky * ky;
    const double rk = rsqrt(k2);                    // 1/k
    const double k = k2 * rk;
    if (!(h <= 0.0) && !(k > 0.0) && !isnan(k)) return RHS_ARGUMENT_OUT_OF_BOUNDS;
    const double kh = k * h;
    const double m = -expm1(-2.0 * kh);             // 1 - exp(-2kh)
    const double q = 1.0 - m;                       // exp(-2kh)
    const double inv_d = 1.0 / (m * (2.0 - m));     // one division for both below
    const double r = m * inv_d;                     // 1 / (2 - m)
    const double th = m * r;                        // tanh(kh)
    const double kh_ch2 = 4.0 * kh * q * r * r;     // kh / cosh(kh)^2
    const double inv_shch = 4.0 * q * (2.0 - m) * inv_d * r;  // 1 / (sinh cosh)
    const double gkt = kG * k * th;
    const double rs = rsqrt(gkt);                   // 1 / sqrt(g k tanh)
    double cg = (kG / 2.0) * (th + kh_ch2) * rs;
    if (h <= 0.0) cg = f64_nan();
    const double f = -0.5 * k * inv_shch * (gkt * rs);
    out[0] = cg * (kx * rk) + cur[0];
    out[1] = cg * (ky * rk) + cur[1];
    out[2] = f * static_cast<double>(hg[1]) - kx * cur[2] - ky * cur[4];
    out[3] = f * static_cast<double>(hg[2]) - kx * cur[3] - ky * cur[5];
    return RHS_OK;
  }
};

// impl System::system (src/wave_ray_path.rs:220-234): errors become NaN.
template <typename Rhs>
__device__ __forceinline__ void system(const BathyDev &b, const CurrentDev &c, const double s[4],
                                       double ds[4]) {
  if (Rhs::odes(b, c, s[0], s[1], s[2], s[3], ds) != RHS_OK) {
    ds[0] = ds[1] = ds[2] = ds[3] = f64_nan();
  }
}

__device__ __forceinline__ bool all_nan4(const double v[4]) {
  return isnan(v[0]) && isnan(v[1]) && isnan(v[2]) && isnan(v[3]);
}

}  // namespace mr
